"""PSP snapshot reader with the interface of ``exptool/io/psp_io.py``
(``Input(filename, comp=None, verbose=0)``: ``.header``, ``.time``,
``.comp``, ``.data``).  The component's records are read into page-locked
memory and de-interleaved by a GPU kernel (exptool_gb300.io.snapshot).

``device=True`` leaves ``.data`` as CUDA tensors (float columns as float64),
ready for the basis pipelines without a host copy; otherwise ``.data`` holds
NumPy arrays of the file's types, as the reference returns.
"""
from __future__ import annotations

from . import snapshot


class Input:
    def __init__(self, filename, comp=None, verbose=0, device=False):
        self.verbose = verbose
        self.filename = filename
        try:
            f = open(filename, "rb")
        except OSError as e:
            raise IOError(f'Failed to open "{filename}"') from e
        with f:
            self.time, self._float_len, self.header = snapshot.read_psp_header(f)
        self.primary_header = dict()
        self.comp = comp
        self.indexing = None
        if comp is not None:
            if comp not in self.header:
                raise IOError("The specified component does not exist.")
            head = self.header[comp]
            self.indexing = snapshot._indexing(head)
            self.data = snapshot.load_psp_component(filename, head, self._float_len, device)

    def _summarise_primary_header(self):
        comps = list(self.header.keys())
        print("Found {} components.".format(len(comps)))
        for n, c in enumerate(comps):
            print("Component {}: {}".format(n, c))

"""SPL (split phase-space) snapshot reader with the interface of
``exptool/io/spl_io.py`` (``Input(filename, comp=None, verbose=0)``; with no
component it prints the component summary and returns).  Sub-files are read
into one page-locked buffer in order and de-interleaved by a GPU kernel
(exptool_gb300.io.snapshot); ``device=True`` as for psp_io.Input.
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
            self.time, self._float_len, self.header, self._subfiles = snapshot.read_spl_header(f)
        self.primary_header = dict()
        self.comp = comp
        if comp is None:
            self._summarise_primary_header()
            return
        if comp not in self.header:
            raise IOError("The specified component does not exist.")
        self.indir = filename.split("SPL")[0]
        self.subfiles = self._subfiles[comp]
        self.nprocs = len(self.subfiles)
        self.indexing = snapshot._indexing(self.header[comp])
        self.data = snapshot.load_spl_component(filename, self.header[comp], self._float_len, self.subfiles, device)

    def _summarise_primary_header(self):
        comps = list(self.header.keys())
        print("Found {} components.".format(len(comps)))
        for n, c in enumerate(comps):
            print("Component {}: {}".format(n, c))

"""EOF table construction on the GPU (``EOFTables(engine="gpu")``: basis
functions by the xt_eof_basis kernel, second moments and tabulation as FP64
device products) against the NumPy engine on the same sample and grid.

Both engines evaluate the same FP64 formulas (the spline of u_nl(ln r), the
normalised Legendre recurrence, forces and density); they differ by the
summation order of the second-moment matrix and the products, so the
eigenvalues agree to ~1e-13 and the tables to the eigenvector rounding
(bound 1e-9 normwise per (m, order) block, relative to the block's largest
entry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gpu_eof_tables_match_numpy(tmp_path):
    from exptool_gb300.basis import eof
    from exptool_gb300.tables.eof_builder import EOFTables
    kw = dict(mmax=3, norder=5, numx=24, numy=20, lmax_sph=10, nmax_sph=8, nsample=20000, seed=7)
    a = EOFTables(engine="numpy", **kw)
    b = EOFTables(engine="gpu", **kw)
    assert np.max(np.abs(b.eigvals - a.eigvals) / np.abs(a.eigvals)) <= 1e-12
    for name in ("pot", "rforce", "zforce", "dens"):
        A, B = getattr(a, name), getattr(b, name)
        for m in range(kw["mmax"] + 1):
            for n in range(kw["norder"]):
                s = np.max(np.abs(A[m, n]))
                assert np.max(np.abs(B[m, n] - A[m, n])) <= 1e-9 * s, (name, m, n)
    # the written cache reads back through the drop-in reader
    path = str(tmp_path / "eof.cache")
    b.write(path)
    potC = eof.parse_eof(path)[0]
    assert np.array_equal(potC, b.pot)

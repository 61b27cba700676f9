"""MatrixMarket round trip of an assembled oracle system (the reference's dump format)."""
import numpy as np

from mrhyde_gb300 import mmio
from tests.cases import oracle_problem


def test_matrix_market_round_trip(tmp_path):
    P = oracle_problem(dict(dim=2, order=1, n=(5, 4), kappa=np.linspace(0.5, 2.0, 20), dirichlet_faces=1))
    u = np.random.default_rng(0).standard_normal(P.ndof)
    r, J = P.assemble(u)
    rp, ci = P.graph()
    mmio.write_csr(tmp_path / "J.mm", rp, ci, J)
    mmio.write_vector(tmp_path / "r.mm", r)
    rp2, ci2, J2 = mmio.read_csr(tmp_path / "J.mm")
    assert np.array_equal(rp2, rp) and np.array_equal(ci2, ci)
    assert np.array_equal(J2, J)  # %.17g round-trips doubles exactly
    assert np.array_equal(mmio.read_vector(tmp_path / "r.mm"), r)
    try:
        import warnings

        import scipy.io
        import scipy.sparse
    except ImportError:
        return
    # an independent reader sees the same matrix: its product with u equals the CSR product of our arrays
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", DeprecationWarning)  # mmread's default return type is changing
        A = scipy.sparse.csr_matrix(scipy.io.mmread(str(tmp_path / "J.mm")))
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    ref = np.bincount(rows, weights=J * u[ci], minlength=len(rp) - 1)
    assert A.nnz == len(J)
    assert np.allclose(A @ u, ref, rtol=1e-13, atol=1e-13 * np.abs(ref).max())

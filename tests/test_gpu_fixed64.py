"""Q1 factored path with exact kappa sums (64-bit fixed point on the integer pipes, each sum rounded once to
FP64; products and residual FMAs in FP64) against the same path with FP64 additions (MRG_ASM_NATIVE_FP64)
and against the oracle.

Cubic cells: the off-diagonal coefficients are +0 (axis neighbours) or one value -|K| (diagonal 4 |K|), so
the kernel sums the scaled conductances RN(|K| kappa_c) exactly and rounds once: J(i, i+off) =
-RN(sum_c RN(|K| kappa_c)) and J(i, i) = 4 RN(sum of the 8), checked bit for bit against that
definition (math.fsum is the correctly rounded sum) and r against its FMA chain in exact rational
arithmetic; within a few ulps of the native products.  Rows outside the fixed point keep the native
products: identical bits.

* integer-valued kappa: every kappa sum is exact in FP64 as well, so both paths form the same sums and
  products -- identical bits;
* lognormal kappa: the exact sums are rounded once where FP64 rounds every partial sum; entries agree to
  a few units in the last place (scaled bound 1e-15), residuals within 1e-13 (scaled), both within 1e-12
  of the oracle;
* rows whose kappa span more than 2^7, or hold a negative kappa, take the FP64 instructions: identical bits.
"""
import numpy as np
import pytest
import torch

from tests.cases import gpu_problem, oracle_problem

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def scaled_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = np.max(np.abs(b)) if b.size else 1.0
    scale = np.maximum(np.abs(b), 1e-3 * m)
    scale[scale == 0] = 1.0
    return float(np.max(np.abs(a - b) / scale))


def _cfg(kappa, n=(9, 7, 6), hi=(1.0, 1.0, 1.0), faces=1 | 2):
    return dict(dim=3, order=1, n=n, hi=hi, kappa=kappa, dirichlet_faces=faces, source=("const", 1.0, 0.0))


def _assemble(G, u, native, fp32=False, jac=True):
    from mrhyde_gb300 import AssemblyManager

    A = AssemblyManager(G)
    ud = torch.tensor(u, device="cuda")
    r = torch.zeros(G.info.n_dofs, dtype=torch.float64, device="cuda")
    J = torch.zeros(G.info.nnz, dtype=torch.float32 if fp32 else torch.float64, device="cuda")
    if jac:
        A.assembleJacRes(ud, r, J, fp32_jacobian=fp32, overwrite=True, native_fp64=native)
    else:
        A.assembleRes(ud, r, overwrite=True, native_fp64=native)
    torch.cuda.synchronize()
    return r.cpu().numpy(), J.cpu().numpy()


def _u(G, seed):
    return np.random.default_rng(seed).uniform(-1, 1, G.info.n_dofs)


@pytest.mark.parametrize("hi", [(1.0, 1.0, 1.0), (1.0, 0.37, 2.5)])
def test_integer_kappa_bit_identical(hi):
    n = (9, 7, 6)
    kap = np.random.default_rng(1).integers(1, 9, n[0] * n[1] * n[2]).astype(np.float64)
    G = gpu_problem(_cfg(kap, n, hi))
    u = _u(G, 2)
    _, J_fx = _assemble(G, u, native=False)
    _, J_nat = _assemble(G, u, native=True)
    assert np.array_equal(J_fx.view(np.uint64), J_nat.view(np.uint64))


@pytest.mark.parametrize("sigma", [0.5, 1.0])
def test_lognormal_kappa_within_ulps_and_oracle(sigma):
    n = (10, 9, 8)
    kap = np.exp(sigma * np.random.default_rng(3).standard_normal(n[0] * n[1] * n[2]))
    cfg = _cfg(kap, n)
    G = gpu_problem(cfg)
    u = _u(G, 4)
    r_fx, J_fx = _assemble(G, u, native=False)
    r_nat, J_nat = _assemble(G, u, native=True)
    assert scaled_err(J_fx, J_nat) <= 1e-15
    assert scaled_err(r_fx, r_nat) <= 1e-13
    r_o, J_o = oracle_problem(cfg).assemble(u)
    assert scaled_err(J_fx, J_o) <= TOL64
    assert scaled_err(r_fx, r_o) <= TOL64
    # residual-only pass forms the same entries in the same order
    r_r, _ = _assemble(G, u, native=False, jac=False)
    assert np.array_equal(r_r, r_fx)


def _fallback_rows(kap, n):
    """Rows whose surrounding cells hold a negative kappa or nonzero kappa more than 2^7 apart (binary
    exponents differing by more than 7)."""
    nx, ny, nz = n
    K = kap.reshape(nz, ny, nx)
    E = np.frexp(np.abs(K))[1]
    rows = []
    for iz in range(nz + 1):
        for iy in range(ny + 1):
            for ix in range(nx + 1):
                cz = [c for c in (iz - 1, iz) if 0 <= c < nz]
                cy = [c for c in (iy - 1, iy) if 0 <= c < ny]
                cx = [c for c in (ix - 1, ix) if 0 <= c < nx]
                v = K[np.ix_(cz, cy, cx)].ravel()
                e = E[np.ix_(cz, cy, cx)].ravel()
                if (v < 0).any() or e.max() - e.min() > 7:
                    rows.append(ix + (nx + 1) * (iy + (ny + 1) * iz))
    return rows


@pytest.mark.parametrize("spoil", ["wide", "negative"])
def test_fallback_rows_bit_identical(spoil):
    n = (6, 6, 6)
    kap = np.exp(0.3 * np.random.default_rng(5).standard_normal(n[0] * n[1] * n[2]))
    if spoil == "wide":
        kap[::7] *= 1e3   # neighbouring kappa ~2^10 apart: those rows take the FP64 instructions
    else:
        kap[11] = -0.5
    G = gpu_problem(_cfg(kap, n))
    u = _u(G, 6)
    r_fx, J_fx = _assemble(G, u, native=False)
    r_nat, J_nat = _assemble(G, u, native=True)
    rp, _ = G.graph()
    rp = rp.cpu().numpy()
    fb = _fallback_rows(kap, n)
    assert fb
    for row in fb:
        assert np.array_equal(J_fx[rp[row]:rp[row + 1]].view(np.uint64), J_nat[rp[row]:rp[row + 1]].view(np.uint64))
        assert r_fx[row] == r_nat[row]
    assert scaled_err(J_fx, J_nat) <= 1e-15
    assert scaled_err(r_fx, r_nat) <= 1e-13


def test_wide_but_exact_kappa_range():
    # kappa spanning 2^6 within rows (exact in the fixed point): still within a few ulps of FP64
    n = (7, 6, 5)
    kap = np.exp2(np.random.default_rng(7).integers(0, 7, n[0] * n[1] * n[2])).astype(np.float64)
    kap *= 1.0 + 0.1 * np.random.default_rng(8).random(kap.size)
    G = gpu_problem(_cfg(kap, n))
    u = _u(G, 9)
    _, J_fx = _assemble(G, u, native=False)
    _, J_nat = _assemble(G, u, native=True)
    nz = J_nat != 0
    rel = np.abs(J_fx[nz] - J_nat[nz]) / np.abs(J_nat[nz])
    assert rel.max() <= 8 * np.finfo(np.float64).eps


def test_mixed_j32_bits_unchanged():
    n = (10, 9, 8)
    kap = np.exp(np.random.default_rng(10).standard_normal(n[0] * n[1] * n[2]))
    G = gpu_problem(_cfg(kap, n))
    u = _u(G, 11)
    r_fx, J_fx = _assemble(G, u, native=False, fp32=True)
    r_nat, J_nat = _assemble(G, u, native=True, fp32=True)
    assert np.array_equal(J_fx, J_nat)
    assert scaled_err(r_fx, r_nat) <= 1e-13


# ---- cubic cells: the axis-neighbour coefficient is +0 and those entries take no FP64 instruction --------
def _axis_slots(G, n):
    """CSR slots of the axis-neighbour entries (column differs from the row in exactly one coordinate)."""
    rp, ci = G.graph()
    rp, ci = rp.cpu().numpy(), ci.cpu().numpy()
    nx, ny = n[0] + 1, n[1] + 1
    rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    d = [np.abs(rows % nx - ci % nx), np.abs(rows // nx % ny - ci // nx % ny), np.abs(rows // (nx * ny) - ci // (nx * ny))]
    return ((d[0] != 0).astype(int) + (d[1] != 0) + (d[2] != 0)) == 1


def _kscale(n, hi):
    """|K| of cubic cells with these sizes: minus the corner entry of an interior row at kappa = 1."""
    G = gpu_problem(_cfg(np.ones(int(np.prod(n))), n, hi, faces=0))
    _, J = _assemble(G, np.zeros(G.info.n_dofs), native=False)
    rp, ci = G.graph()
    rp, ci = rp.cpu().numpy(), ci.cpu().numpy()
    nx, ny = n[0] + 1, n[1] + 1
    row = 1 + nx * (1 + ny)  # node (1, 1, 1)
    assert ci[rp[row]] == 0  # its first column: node (0, 0, 0), the corner (-1, -1, -1)
    return -J[rp[row]]


def _emulate_cube(kap, n, ks, u, b):
    """J and r of the cubic-cell path on exact-sum rows, from the definition (None for other rows)."""
    import math
    from fractions import Fraction

    nx, ny, nz = n
    K = kap.reshape(nz, ny, nx)
    Ks = K * ks  # RN(kappa |K|): the IEEE multiply
    NX, NY, NZ = nx + 1, ny + 1, nz + 1
    Jrows, rrows = {}, {}
    for iz in range(NZ):
        for iy in range(NY):
            for ix in range(NX):
                cells = {}
                for c in (0, 1):
                    for bb in (0, 1):
                        for a in (0, 1):
                            cx, cy, cz = ix - 1 + a, iy - 1 + bb, iz - 1 + c
                            if 0 <= cx < nx and 0 <= cy < ny and 0 <= cz < nz:
                                cells[(a, bb, c)] = Ks[cz, cy, cx]
                vals = [v for v in cells.values() if v != 0]
                e = [math.frexp(v)[1] for v in vals]
                if any(v < 0 for v in vals) or (vals and max(e) - min(e) > 7):
                    continue  # fallback row
                row, acc = [], Fraction(b[ix + NX * (iy + NY * iz)])
                for dz in (-1, 0, 1):
                    for dy in (-1, 0, 1):
                        for dx in (-1, 0, 1):
                            if not (0 <= ix + dx < NX and 0 <= iy + dy < NY and 0 <= iz + dz < NZ):
                                continue
                            nzc = (dx != 0) + (dy != 0) + (dz != 0)
                            if nzc == 1:
                                row.append(0.0)
                                continue
                            # the cells containing both nodes: a = 0 (below) or 1 (above) along each axis
                            sh = [v for (a, bb, c), v in cells.items()
                                  if (dx == 0 or a == (dx > 0)) and (dy == 0 or bb == (dy > 0)) and (dz == 0 or c == (dz > 0))]
                            ssum = math.fsum(sh)
                            ent = 4.0 * ssum if nzc == 0 else -ssum
                            row.append(ent)
                            uv = u[ix + dx + NX * (iy + dy + NY * (iz + dz))]
                            acc = Fraction(float(-Fraction(ent) * Fraction(uv) + acc))  # one FMA
                n_ = ix + NX * (iy + NY * iz)
                Jrows[n_] = np.array(row)
                rrows[n_] = float(acc)
    return Jrows, rrows


@pytest.mark.parametrize("kind", ["integer", "lognormal", "wide"])
def test_cube_scaled_sums_exact(kind):
    n = (7, 7, 7)
    hi = (0.7, 0.7, 0.7)
    rng = np.random.default_rng(21)
    if kind == "integer":
        kap = rng.integers(1, 9, 343).astype(np.float64)
    elif kind == "lognormal":
        kap = np.exp(rng.standard_normal(343))
    else:  # some rows outside the fixed point
        kap = np.exp(0.3 * rng.standard_normal(343))
        kap[::11] *= 1e3
    ks = _kscale(n, hi)
    G = gpu_problem(_cfg(kap, n, hi, faces=0))
    u = _u(G, 22)
    b, _ = _assemble(G, np.zeros(G.info.n_dofs), native=False, jac=False)
    r_fx, J_fx = _assemble(G, u, native=False)
    r_nat, J_nat = _assemble(G, u, native=True)
    Jrows, rrows = _emulate_cube(kap, n, ks, u, b)
    rp, _ = G.graph()
    rp = rp.cpu().numpy()
    assert len(Jrows) > 0
    for row, Je in Jrows.items():
        assert np.array_equal(J_fx[rp[row]:rp[row + 1]].view(np.uint64), Je.view(np.uint64)), row
        assert r_fx[row] == rrows[row], row
    fb = [k for k in range(G.info.n_dofs) if k not in Jrows]
    if kind == "wide":
        assert fb
    for row in fb:  # native products
        assert np.array_equal(J_fx[rp[row]:rp[row + 1]].view(np.uint64), J_nat[rp[row]:rp[row + 1]].view(np.uint64))
        assert r_fx[row] == r_nat[row]
    nz = J_nat != 0
    assert np.max(np.abs(J_fx[nz] - J_nat[nz]) / np.abs(J_nat[nz])) <= 4 * np.finfo(np.float64).eps
    assert scaled_err(r_fx, r_nat) <= 1e-13
    r_r, _ = _assemble(G, u, native=False, jac=False)
    assert np.array_equal(r_r, r_fx)


@pytest.mark.parametrize("kind", ["integer", "lognormal"])
def test_cube_axis_entries(kind):
    n = (8, 8, 8)
    rng = np.random.default_rng(12)
    kap = rng.integers(1, 9, 512).astype(np.float64) if kind == "integer" else np.exp(rng.standard_normal(512))
    cfg = _cfg(kap, n, hi=(0.5, 0.5, 0.5))
    G = gpu_problem(cfg)
    u = _u(G, 13)
    r_fx, J_fx = _assemble(G, u, native=False)
    r_nat, J_nat = _assemble(G, u, native=True)   # every product a DMUL
    ax = _axis_slots(G, n)
    assert ax.sum() > 0 and np.all(J_fx[ax].view(np.uint64) == 0)  # +0
    assert np.array_equal(J_fx[ax].view(np.uint64), J_nat[ax].view(np.uint64))
    # the other entries: exact sums of scaled conductances, within a few ulps of the native products
    assert scaled_err(J_fx, J_nat) <= 1e-15
    assert scaled_err(r_fx, r_nat) <= 1e-13
    r_o, J_o = oracle_problem(cfg).assemble(u)
    assert scaled_err(J_fx, J_o) <= TOL64
    assert scaled_err(r_fx, r_o) <= TOL64
    r_r, _ = _assemble(G, u, native=False, jac=False)
    assert np.array_equal(r_r, r_fx)


def test_cube_signed_and_nonfinite_entries():
    # negative kappa (zero entries with the sign of S), kappa near the top of the range (sums overflow to
    # inf: +0 * inf is NaN) and a non-finite u: those rows take the native products (the same values as
    # the plain FP64 instructions); the others agree to a few ulps
    n = (6, 6, 6)
    kap = np.random.default_rng(14).integers(1, 9, 216).astype(np.float64)  # exact sums on both paths
    kap[17] = -12.5
    kap[100] = 1.5e308
    kap[101] = 1.2e308
    cfg = _cfg(kap, n)
    G = gpu_problem(cfg)
    u = _u(G, 15)
    u[150] = np.inf
    u[40] = np.nan
    r_fx, J_fx = _assemble(G, u, native=False)
    r_nat, J_nat = _assemble(G, u, native=True)
    fin = ~np.isnan(J_nat)
    assert np.array_equal(np.isnan(J_fx), ~fin)
    assert np.array_equal(np.isnan(r_fx), np.isnan(r_nat))
    assert np.array_equal(np.isinf(J_fx), np.isinf(J_nat)) and np.array_equal(np.isinf(r_fx), np.isinf(r_nat))
    rp, _ = G.graph()
    rp = rp.cpu().numpy()
    fb = _fallback_rows(kap, n)
    for row in fb:  # the native products (NaN entries compared as NaN, whatever their payload)
        a, c = J_fx[rp[row]:rp[row + 1]], J_nat[rp[row]:rp[row + 1]]
        m = ~np.isnan(c)
        assert np.array_equal(np.isnan(a), ~m) and np.array_equal(a[m].view(np.uint64), c[m].view(np.uint64))
        assert np.array_equal(r_fx[row], r_nat[row], equal_nan=True)
    ok = np.isfinite(J_nat) & (J_nat != 0)
    assert np.max(np.abs(J_fx[ok] - J_nat[ok]) / np.abs(J_nat[ok])) <= 4 * np.finfo(np.float64).eps
    ax = _axis_slots(G, n)
    assert (np.signbit(J_fx[ax & fin])).any() and (~np.signbit(J_fx[ax & fin])).any()


def test_cube_mixed_j32_unchanged_and_residual():
    n = (8, 8, 8)
    kap = np.exp(np.random.default_rng(16).standard_normal(512))
    cfg = _cfg(kap, n, hi=(0.5, 0.5, 0.5))
    G = gpu_problem(cfg)
    u = _u(G, 17)
    r_fx, J_fx = _assemble(G, u, native=False, fp32=True)
    r_nat, J_nat = _assemble(G, u, native=True, fp32=True)
    assert np.array_equal(J_fx.view(np.uint32), J_nat.view(np.uint32))
    assert scaled_err(r_fx, r_nat) <= 1e-13
    r64, _ = _assemble(G, u, native=False)
    assert scaled_err(r_fx, r64) <= 1e-13
    u[77] = np.nan
    r_fx, _ = _assemble(G, u, native=False, fp32=True)
    r_nat, _ = _assemble(G, u, native=True, fp32=True)
    assert np.array_equal(np.isnan(r_fx), np.isnan(r_nat)) and np.isnan(r_fx).sum() > 1


@pytest.mark.parametrize("hi", [(0.8, 0.7, 0.6), (1.0, 0.37, 2.5), (1e4, 1e4, 1e4)])  # cubic cells, boxes, huge h
def test_residual_only_corner_products_bit_identical(hi):
    # box cells: the residual-only pass forms the corner products K * kappa on the integer pipes: the same
    # bits as the FP64 multiply of the Jacobian pass and of the native path, including zero kappa (a -0
    # product), a block of kappa near the top of the exact-sum range (rows inside it keep the integer
    # products) and, on the coarse grid (h = 1250), products that would overflow (those rows take the
    # multiply: inf).  Cubic cells (h = 0.1) sum scaled conductances in both passes: the residual-only pass
    # gives the Jacobian pass's bits, and the native path's to a few ulps of the row's terms
    n = (8, 7, 6)
    kap = np.random.default_rng(18).integers(1, 9, n[0] * n[1] * n[2]).astype(np.float64)
    K = kap.reshape(n[2], n[1], n[0])
    K[1:4, 2:5, 3:6] = 1.7e306 * (1.0 + np.arange(27).reshape(3, 3, 3) % 3)
    K[4, 5, 6] = 0.0
    K[0, 0, 0] = 1e-300
    G = gpu_problem(_cfg(kap, n, hi))
    u = _u(G, 19)
    r_res, _ = _assemble(G, u, native=False, jac=False)
    r_jr, _ = _assemble(G, u, native=False)
    r_nat, _ = _assemble(G, u, native=True, jac=False)
    assert np.array_equal(r_res, r_jr, equal_nan=True)
    if hi[0] == 0.8:
        assert np.array_equal(np.isnan(r_res), np.isnan(r_nat)) and scaled_err(r_res, r_nat) <= 1e-13
    else:
        assert np.array_equal(r_res, r_nat, equal_nan=True)
    if hi[0] > 100:
        assert np.isinf(r_res).any() or np.isnan(r_res).any()
    kap2 = np.exp(np.random.default_rng(20).standard_normal(n[0] * n[1] * n[2]))
    G2 = gpu_problem(_cfg(kap2, n, hi))
    r_res, _ = _assemble(G2, u, native=False, jac=False)
    r_jr, _ = _assemble(G2, u, native=False)
    assert np.array_equal(r_res, r_jr)

"""The Gauss-Newton operators through the C ABI (afx_gn_*) against the CPU oracle, on one
frame of the small non-rigid case with the reference's constants (K = 6 skinning, K_reg = 4)
and with the workload's (K = 4, K_reg = 8): residuals and J^T J bit-exact, J^T r to rounding
(the GPU sums rows in a fixed butterfly, the oracle in sequence), the PCG solution against the
oracle's FP64 PCG, and the transform update bit-exact."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402
from _gn_system import gn_system  # noqa: E402

pytestmark = pytest.mark.gpu


def cu(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return (t.to(dtype) if dtype is not None else t).cuda()


_system = gn_system


@pytest.mark.parametrize("k,kreg", [(6, 4), (4, 8)])
def test_gauss_newton_operators_match_oracle(k, kreg):
    from volumefusion_gb300 import af
    s = _system(k, kreg)
    n, m, nc = len(s["nodes"]), len(s["mesh"]), len(s["corr"])
    assert n > 10 and nc > 100
    # oracle
    rd = O.residual_depth(s["corr"], s["warped"], s["v1"], s["n1"], s["lam_d"])
    rr = O.residual_reg(s["nodes"], s["T"], s["gidx"], s["lam_r"])
    A, b, _ = O.assemble(s["corr"], s["mesh"], s["midx"], s["mw"], s["n1"], s["lam_d"], s["nodes"], s["gidx"],
                         s["lam_r"], rd, rr)
    x_o, _ = O.pcg(A, b, 10)
    # GPU
    g = af.GaussNewtonSystem(m + 16, n + 8, k, kreg)
    cnt = lambda v: cu(np.array([v], np.int32))  # noqa: E731
    g.build(cu(s["mesh"]), cnt(m), cu(s["midx"].view(np.int32)), cu(s["mw"]), cu(s["corr"]), cnt(nc), cu(s["v1"]),
            cu(s["n1"]), cu(s["warped"]), cu(s["nodes"]), cu(s["T"]), cnt(n), cu(s["gidx"].view(np.int32)),
            s["lam_d"], s["lam_r"])
    jtj, jtr, grd, grr = g.export(n, nc)
    assert np.array_equal(grd.cpu().numpy(), rd)
    assert np.array_equal(grr.cpu().numpy(), rr)
    assert np.array_equal(jtj.cpu().numpy(), A)
    jb = jtr.cpu().numpy()
    assert np.abs(jb - b).max() <= 1e-5 * max(1.0, np.abs(b).max())
    # The system is stiff (condition number ~5e6 here: the regulariser is a graph Laplacian), so
    # FP32 and FP64 Krylov iterates part by up to ~kappa * eps.  Converged: the true residual
    # |b - A x| / |b| reaches FP32 level and x is within a few percent of the exact FP64 solve.
    A64, b64 = A.astype(np.float64), b.astype(np.float64)
    x_exact = np.linalg.solve(A64, b64)
    xc = g.solve(400, tol=1e-7)[:6 * n].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(b64 - A64 @ xc) <= 1e-4 * np.linalg.norm(b64)
    assert np.linalg.norm(xc - x_exact) <= 5e-2 * np.linalg.norm(x_exact)
    # ten iterations (the workload's setting) against the oracle's FP64 PCG
    x = g.solve(10)[:6 * n].cpu().numpy()
    assert np.linalg.norm(x - x_o) <= 3e-2 * np.linalg.norm(x_o)
    # transform update with the same x
    Tg = cu(s["T"])
    af.runUpdateTransformsKernel(Tg, cu(x), cnt(n))
    assert np.array_equal(Tg.cpu().numpy(), O.update_transforms(s["T"], x))
    g.close()


def test_global_memory_pcg_on_a_tiled_system():
    """The PCG path for graphs too large for distributed shared memory (more than 1024 nodes), on
    a well-posed system of that size: 40 copies of the small system with disjoint node, vertex and
    pixel indices (the copies share coordinates, which the assembly never searches), so J^T J is
    block-diagonal with 40 equal blocks and every copy's PCG iterates are the single system's.
    Each copy's solution matches the oracle's FP64 PCG of the single system as the small-system
    test does, and all copies agree with each other."""
    from volumefusion_gb300 import af
    s = _system(4, 8)
    n, m, nc = len(s["nodes"]), len(s["mesh"]), len(s["corr"])
    copies = 40
    assert n * copies > 1024
    P = s["v1"].shape[0] * s["v1"].shape[1]
    inval = np.uint32(0xFFFFFFFF)

    def offset(idx, step):
        out = [np.where(idx == inval, inval, idx + np.uint32(c * step)).astype(np.uint32) for c in range(copies)]
        return np.concatenate(out)

    mesh = np.tile(s["mesh"], (copies, 1))
    midx = offset(s["midx"], n)
    mw = np.tile(s["mw"], (copies, 1))
    corr = np.concatenate([s["corr"] + np.array([c * m, c * P], np.int32) for c in range(copies)])
    v1 = np.tile(s["v1"].reshape(-1, 3), (copies, 1))
    n1 = np.tile(s["n1"].reshape(-1, 3), (copies, 1))
    warped = np.tile(s["warped"], (copies, 1))
    nodes = np.tile(s["nodes"], (copies, 1))
    T = np.tile(s["T"], (copies, 1))
    gidx = offset(s["gidx"], n)
    # oracle: the single system
    rd = O.residual_depth(s["corr"], s["warped"], s["v1"], s["n1"], s["lam_d"])
    rr = O.residual_reg(s["nodes"], s["T"], s["gidx"], s["lam_r"])
    A, b, _ = O.assemble(s["corr"], s["mesh"], s["midx"], s["mw"], s["n1"], s["lam_d"], s["nodes"], s["gidx"],
                         s["lam_r"], rd, rr)
    x_o, _ = O.pcg(A, b, 10)
    N = n * copies
    g = af.GaussNewtonSystem(m * copies + 16, N + 8, 4, 8)
    cnt = lambda v: cu(np.array([v], np.int32))  # noqa: E731
    g.build(cu(mesh), cnt(m * copies), cu(midx.view(np.int32)), cu(mw), cu(corr), cnt(nc * copies), cu(v1), cu(n1),
            cu(warped), cu(nodes), cu(T), cnt(N), cu(gidx.view(np.int32)), s["lam_d"], s["lam_r"])
    x = g.solve(10)[:6 * N].cpu().numpy().reshape(copies, 6 * n)
    for c in range(copies):
        assert np.array_equal(x[c], x[0]), c
        assert np.linalg.norm(x[c] - x_o) <= 3e-2 * np.linalg.norm(x_o)
    # the same solve through the shared-memory path (the single system): the two paths sum their
    # SpMV rows and dot products in different orders, so a step size can round to a neighbouring
    # binary32 value.  This system is stiff (condition number ~5e6): one ulp of one early step size
    # moves ten binary32 PCG iterations by several 1e-3 relative, up to 2.2e-2 depending on the SpMV's
    # summation order (tests/test_pcg_sensitivity.py).  Both paths are held to the oracle's binary64
    # PCG at 3e-2 above and in the test before; here they agree within the same.
    g1 = af.GaussNewtonSystem(m + 16, n + 8, 4, 8)
    g1.build(cu(s["mesh"]), cnt(m), cu(s["midx"].view(np.int32)), cu(s["mw"]), cu(s["corr"]), cnt(nc), cu(s["v1"]),
             cu(s["n1"]), cu(s["warped"]), cu(s["nodes"]), cu(s["T"]), cnt(n), cu(s["gidx"].view(np.int32)),
             s["lam_d"], s["lam_r"])
    x1 = g1.solve(10)[:6 * n].cpu().numpy()
    assert np.linalg.norm(x1 - x_o) <= 3e-2 * np.linalg.norm(x_o)
    assert np.linalg.norm(x[0] - x1) <= 3e-2 * np.linalg.norm(x1)
    g.close()
    g1.close()

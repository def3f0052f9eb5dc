"""Why the GPU's ten PCG iterations are compared with the oracle's binary64 PCG within 3e-2 relative
(tests/test_gauss_newton_gpu.py, tests/test_cpp_surface_gpu.py), shown on the CPU with the system
those tests solve (small non-rigid case, K = 4, K_reg = 8; condition number ~5e6).

The GPU keeps the PCG vectors in binary32, accumulates its block SpMV in binary32, and forms each
step size alpha = r.z / p.Ap as a binary32 quotient of totals summed in higher precision
(double-binary32).  Any change in how those totals or the SpMV rows are summed -- another tree,
another arithmetic, another path -- can round a step size to a neighbouring binary32 value.  Here a
binary32 restatement of the block-Jacobi PCG is run with one step size moved by one ulp: on this
system that alone moves x by several 1e-3 relative (up to 2.2e-2 with another summation order of the
SpMV rows), so two correct binary32 solvers part by up to that much, while each stays within a few
1e-3 of the binary64 iterates."""
import numpy as np

from _gn_system import assembled, gn_system
from oracle import pyoracle as O

f32 = np.float32


def _pcg32(A, b, iters=10, bump=None):
    # binary32 arithmetic as the GPU's: every product rounded, the SpMV rows and the 6x6
    # preconditioner products accumulated in binary32 (numpy's fixed pairwise order for the rows,
    # sequential for the 6x6), the dot products in binary64
    n = len(b) // 6
    A = np.ascontiguousarray(A, f32)
    minv = np.stack([np.linalg.inv(A[6 * i:6 * i + 6, 6 * i:6 * i + 6].astype(np.float64)) for i in range(n)]).astype(f32)

    def precond(r):
        rb = r.reshape(n, 6)
        z = np.zeros((n, 6), f32)
        for q in range(6):
            z = (z + minv[:, :, q] * rb[:, q:q + 1]).astype(f32)
        return z.reshape(-1)

    def spmv(p):
        return (A * p[None, :]).sum(axis=1, dtype=f32)

    def dot(x, y):
        return np.dot(x.astype(np.float64), y.astype(np.float64))

    x = np.zeros(len(b), f32)
    r = b.astype(f32).copy()
    z = precond(r)
    p = z.copy()
    rz = dot(r, z)
    beta = f32(0)
    for it in range(iters):
        if it:
            p = (z + beta * p).astype(f32)
        ap = spmv(p)
        alpha = f32(rz / dot(p, ap))
        if bump == it:
            alpha = np.nextafter(alpha, f32(np.inf))
        x = (x + alpha * p).astype(f32)
        r = (r - alpha * ap).astype(f32)
        z = precond(r)
        rz_new = dot(r, z)
        beta = f32(rz_new / rz)
        rz = rz_new
    return x


def test_one_ulp_of_a_step_size_moves_ten_pcg_iterations_by_several_1e3():
    A, b = assembled(gn_system(4, 8))
    x0 = _pcg32(A, b)
    x_o, _ = O.pcg(A, b, 10)
    rel = lambda d, ref: float(np.linalg.norm(d) / np.linalg.norm(ref))  # noqa: E731
    # the binary32 iterates stay close to the binary64 ones when nothing is perturbed (8.3e-3 here)
    assert rel(x0 - x_o, x_o) < 3e-2
    moved = [rel(_pcg32(A, b, bump=k) - x0, x0) for k in range(10)]
    # one ulp (6e-8 relative) of one early step size moves x by more than 3e-3 (6.8e-3 here)
    assert max(moved) > 3e-3, moved
    # the last step size only scales the last update
    assert moved[-1] < 1e-4, moved

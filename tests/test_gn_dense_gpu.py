"""The reference's dense Gauss-Newton operators on the GPU (afx_fill_j_*, afx_fill_r_*,
afx_jtj_contrib_*, afx_multiply_*, afx_fill_jtj / afx_fill_jtr; src/MotionOptimization.cu) driven in
the reference caller's order (src/VolumeFusion.cu:454-646, its thrust sort + reduce_by_key steps
done here on the host as stable sorts and sequential binary32 sums), against the reference's own
kernels run on the host (tests/golden/ref_kernels.npz): the residuals, J^T J and J^T r bit for bit.
Then afx_lu_solve (linearSolverLUStable) on that system, and its singular-matrix status."""
import ctypes as C
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import pyoracle as O  # noqa: E402

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def _g():
    with np.load(os.path.join(HERE, "golden", "ref_kernels.npz")) as z:
        return {k: z[k] for k in z.files}


def _dev(a, dtype=None):
    a = np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype))
    return torch.from_numpy(a.copy()).cuda()


def _ok(rc, what):
    from volumefusion_gb300._lib import check
    check(rc, what)


def _system(G):
    from volumefusion_gb300._lib import lib
    L = lib()
    K, KR = 6, 4
    d1, v1, n1, _ = O.frame_prep(G["mm1"], G["K"])
    lam_d, lam_r = np.float32(1.0), np.float32(np.sqrt(200.0))
    corr, nodes, T, gidx = G["corr"], G["nodes"], G["T"], G["gidx"]
    Cn, n = len(corr), len(nodes)
    hD, hR = Cn, n * KR * 3
    rows_total = hD + hR
    J = torch.zeros((rows_total, n, 6), dtype=torch.float32, device="cuda")
    r = torch.zeros(rows_total, dtype=torch.float32, device="cuda")
    corr_d, mesh_d = _dev(corr, np.int32), _dev(G["mesh"], np.float32)
    midx_d, mw_d = _dev(G["midx"], np.uint32), _dev(G["mw"], np.float32)
    n1_d, v1_d = _dev(n1.reshape(-1, 3), np.float32), _dev(v1.reshape(-1, 3), np.float32)
    warped_d, nodes_d = _dev(G["warped"], np.float32), _dev(nodes, np.float32)
    T_d, gidx_d = _dev(T, np.float32), _dev(gidx, np.uint32)
    s = torch.cuda.current_stream().cuda_stream
    _ok(L.afx_fill_j_depth(J.data_ptr(), float(lam_d), hD, n, corr_d.data_ptr(), Cn, mesh_d.data_ptr(),
                           midx_d.data_ptr(), mw_d.data_ptr(), K, n1_d.data_ptr(), s), "afx_fill_j_depth")
    _ok(L.afx_fill_r_depth(r.data_ptr(), float(lam_d), corr_d.data_ptr(), Cn, warped_d.data_ptr(), v1_d.data_ptr(),
                           n1_d.data_ptr(), s), "afx_fill_r_depth")
    _ok(L.afx_fill_r_mreg(r.data_ptr() + 4 * hD, float(lam_r), nodes_d.data_ptr(), T_d.data_ptr(), n,
                          gidx_d.data_ptr(), KR, s), "afx_fill_r_mreg")
    _ok(L.afx_fill_j_mreg(J.data_ptr() + 4 * 6 * hD * n, float(lam_r), hR, n, nodes_d.data_ptr(), n,
                          gidx_d.data_ptr(), KR, s), "afx_fill_j_mreg")
    max_pairs = hD * (K * (K - 1) // 2 + K) + hR * 3
    max_elems = hD * K + hR * 2
    pairs = torch.zeros((max_pairs, 2), dtype=torch.int32, device="cuda")
    prow = torch.zeros(max_pairs, dtype=torch.int32, device="cuda")
    elems = torch.zeros((max_elems, 2), dtype=torch.int32, device="cuda")
    cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
    ws_n = max(L.afx_jtj_contrib_workspace_size(Cn), L.afx_jtj_contrib_workspace_size(n))
    ws = torch.empty(ws_n, dtype=torch.uint8, device="cuda")
    _ok(L.afx_jtj_contrib_depth(pairs.data_ptr(), prow.data_ptr(), cnt.data_ptr(), elems.data_ptr(),
                                cnt.data_ptr() + 4, corr_d.data_ptr(), Cn, midx_d.data_ptr(), mw_d.data_ptr(), K,
                                ws.data_ptr(), ws_n, s), "afx_jtj_contrib_depth")
    _ok(L.afx_jtj_contrib_mreg(pairs.data_ptr(), prow.data_ptr(), hD, cnt.data_ptr(), elems.data_ptr(),
                               cnt.data_ptr() + 4, n, gidx_d.data_ptr(), KR, ws.data_ptr(), ws_n, s),
        "afx_jtj_contrib_mreg")
    npairs, nelems = (int(v) for v in cnt.cpu().numpy())
    P = pairs[:npairs].cpu().numpy()
    R = prow[:npairs].cpu().numpy()
    E = elems[:nelems].cpu().numpy()
    # thrust::sort_by_key on the pairs, restated as a stable lexicographic sort
    order = np.lexsort((P[:, 1], P[:, 0]))
    sp, sr = _dev(P[order]), _dev(R[order])
    prod = torch.empty((npairs, 36), dtype=torch.float32, device="cuda")
    _ok(L.afx_multiply_jtj_pairs(prod.data_ptr(), sp.data_ptr(), sr.data_ptr(), npairs, J.data_ptr(), n, s),
        "afx_multiply_jtj_pairs")
    prod = prod.cpu().numpy()
    keys = P[order]
    coords, sums = [], []
    for i in range(npairs):  # reduce_by_key: sequential binary32 sums
        if coords and (coords[-1] == keys[i]).all():
            sums[-1] = sums[-1] + prod[i]
        else:
            coords.append(keys[i])
            sums.append(prod[i].copy())
    eorder = np.argsort(E[:, 1], kind="stable")
    se = _dev(E[eorder])
    eprod = torch.empty((nelems, 6), dtype=torch.float32, device="cuda")
    _ok(L.afx_multiply_jtr_elems(eprod.data_ptr(), se.data_ptr(), nelems, J.data_ptr(), r.data_ptr(), n, s),
        "afx_multiply_jtr_elems")
    eprod = eprod.cpu().numpy()
    ekeys = E[eorder]
    ecoords, esums = [], []
    for i in range(nelems):
        if ecoords and ecoords[-1][1] == ekeys[i][1]:
            esums[-1] = esums[-1] + eprod[i]
        else:
            ecoords.append(ekeys[i])
            esums.append(eprod[i].copy())
    W = 6 * n
    # the device copies are held in names until the kernels have run: a temporary's memory would go
    # back to the allocator (and to the next copy) while the launch that reads it is still queued
    c_d, s_d = _dev(np.array(coords, np.int32)), _dev(np.array(sums, np.float32))
    ec_d, es_d = _dev(np.array(ecoords, np.int32)), _dev(np.array(esums, np.float32))
    jtj = torch.eye(W, dtype=torch.float32, device="cuda")  # runInitIdentityKernel
    _ok(L.afx_fill_jtj(jtj.data_ptr(), c_d.data_ptr(), s_d.data_ptr(), len(coords), W, s), "afx_fill_jtj")
    jtr = torch.zeros(W, dtype=torch.float32, device="cuda")
    _ok(L.afx_fill_jtr(jtr.data_ptr(), ec_d.data_ptr(), es_d.data_ptr(), len(ecoords), s), "afx_fill_jtr")
    torch.cuda.synchronize()
    return r.cpu().numpy(), jtj, jtr, (P, R, E, hD)


def test_dense_operators_match_reference_kernels():
    G = _g()
    r, jtj, jtr, (P, R, E, hD) = _system(G)
    assert np.array_equal(r, G["residuals"])
    assert np.array_equal(jtj.cpu().numpy(), G["jtj"])
    assert np.array_equal(jtr.cpu().numpy(), G["jtr"])
    # the lists come out in row order: pairs of row c before those of row c + 1
    assert np.all(np.diff(R.astype(np.int64)) >= 0) and np.all(P[:, 0] <= P[:, 1])
    assert R.max() >= hD  # regularisation rows follow the depth rows


def test_lu_solve():
    from volumefusion_gb300._lib import lib
    L = lib()
    G = _g()
    _, jtj, jtr, _ = _system(G)
    n = jtj.shape[0]
    A = jtj.t().contiguous()  # column-major, as handed to cusolverDnSgetrf
    x = torch.empty(n, dtype=torch.float32, device="cuda")
    piv = torch.empty(n, dtype=torch.int32, device="cuda")
    wsn = L.afx_lu_solve_workspace_size(n, n)
    ws = torch.empty(wsn, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    from volumefusion_gb300 import af
    assert af.linearSolverLUStable(None, n, A, n, jtr, piv, x)
    A64 = G["jtj"].astype(np.float64)
    b64 = G["jtr"].astype(np.float64)
    x64 = np.linalg.solve(A64, b64)
    xs = x.cpu().numpy().astype(np.float64)
    # backward error of a binary32 LU; the forward error is that of LAPACK's binary32 LU (sgetrf /
    # sgetrs, what cuSOLVER computes) on this system, within a small factor
    assert np.linalg.norm(A64 @ xs - b64) <= 1e-4 * np.linalg.norm(b64)
    sla = pytest.importorskip("scipy.linalg")
    x32 = sla.lu_solve(sla.lu_factor(G["jtj"].astype(np.float32)), G["jtr"].astype(np.float32)).astype(np.float64)
    assert np.linalg.norm(xs - x64) <= 4 * np.linalg.norm(x32 - x64) + 1e-6 * np.linalg.norm(x64)
    p = piv.cpu().numpy()
    assert p.min() >= 1 and p.max() <= n
    # the input matrix is left as it was
    assert torch.equal(A, jtj.t().contiguous())
    # a matrix with a zero column: getrf's info != 0 becomes AFX_ERR_SINGULAR
    S = torch.eye(8, dtype=torch.float32, device="cuda")
    S[:, 5] = 0
    b = torch.ones(8, dtype=torch.float32, device="cuda")
    x8 = torch.empty(8, dtype=torch.float32, device="cuda")
    p8 = torch.empty(8, dtype=torch.int32, device="cuda")
    w8 = L.afx_lu_solve_workspace_size(8, 8)
    ws8 = torch.empty(w8, dtype=torch.uint8, device="cuda")
    rc = L.afx_lu_solve(x8.data_ptr(), S.data_ptr(), 8, 8, b.data_ptr(), p8.data_ptr(), ws8.data_ptr(), w8, s)
    assert rc == 4  # AFX_ERR_SINGULAR
    assert af.linearSolverLUStable(None, 8, S, 8, b, p8, x8) is False


def test_dense_operators_python_names():
    """The same sequence through volumefusion_gb300.af's reference-named wrappers gives the same
    residuals and J^T J (the first two steps and the J^T J scatter)."""
    from volumefusion_gb300 import af
    G = _g()
    r_ref, jtj_ref, _, (P, R, E, hD) = _system(G)
    K = G["K"]
    d1, v1, n1, _ = O.frame_prep(G["mm1"], K)
    corr, nodes, T, gidx = G["corr"], G["nodes"], G["T"], G["gidx"]
    Cn, n = len(corr), len(nodes)
    hR = n * 4 * 3
    J = torch.zeros((hD + hR, n, 6), dtype=torch.float32, device="cuda")
    r = torch.zeros(hD + hR, dtype=torch.float32, device="cuda")
    corr_d, mesh_d = _dev(corr, np.int32), _dev(G["mesh"], np.float32)
    midx_d, mw_d = _dev(G["midx"], np.uint32), _dev(G["mw"], np.float32)
    n1_d, v1_d = _dev(n1.reshape(-1, 3), np.float32), _dev(v1.reshape(-1, 3), np.float32)
    warped_d, nodes_d = _dev(G["warped"], np.float32), _dev(nodes, np.float32)
    T_d, gidx_d = _dev(T, np.float32), _dev(gidx, np.uint32)
    af.runFill_J_DepthKernel(J, 1.0, hD, n, corr_d, Cn, mesh_d, midx_d, mw_d, v1_d, n1_d)
    af.runFill_r_DepthKernel(r, 1.0, corr_d, Cn, warped_d, v1_d, n1_d)
    af.runFill_r_MRegKernel(r[hD:], float(np.float32(np.sqrt(200.0))), nodes_d, T_d, n, gidx_d)
    af.runFill_J_MRegKernel(J[hD:], float(np.float32(np.sqrt(200.0))), hR, n, nodes_d, T_d, n, gidx_d)
    assert np.array_equal(r.cpu().numpy(), r_ref)
    pairs = torch.zeros((len(P) + 8, 2), dtype=torch.int32, device="cuda")
    rows = torch.zeros(len(P) + 8, dtype=torch.int32, device="cuda")
    elems = torch.zeros((len(E) + 8, 2), dtype=torch.int32, device="cuda")
    npairs = torch.zeros(1, dtype=torch.int32, device="cuda")
    nelems = torch.zeros(1, dtype=torch.int32, device="cuda")
    af.runComputeJTJAndJTrContribJDepthKernel(pairs, rows, npairs, elems, nelems, corr_d, Cn, midx_d, mw_d)
    af.runComputeJTJAndJTrContribJMRegKernel(pairs, rows, hD, npairs, elems, nelems, n, gidx_d)
    assert int(npairs.item()) == len(P) and int(nelems.item()) == len(E)
    assert np.array_equal(pairs[:len(P)].cpu().numpy(), P) and np.array_equal(rows[:len(P)].cpu().numpy(), R)

"""Serving many sessions on one GPU (afx_server_*): a session's results are the same alone and
in a mix of concurrent sessions, results come back in order per session, and admission follows
the memory budget."""
import numpy as np
import pytest


def _mix_configs():
    from volumefusion_gb300 import configs, synth
    a = configs.small_nonrigid(n_frames=8)
    b = configs.small_nonrigid(n_frames=8, dims=(48, 48, 48), voxel=0.011)
    c = configs.small_nonrigid(n_frames=8)
    c["graph_radius"] = 0.04
    K = c["K"]
    sphere = [synth.moving_sphere_frame(i, n_frames=8, width=c["width"], height=c["height"], fx=float(K[0, 0]),
                                        fy=float(K[1, 1]), cx=float(K[0, 2]), cy=float(K[1, 2]))[0] for i in range(8)]
    return [(a, configs.small_frames(a)), (b, configs.small_frames(b)[::-1]), (c, sphere)]


def _drain(server, expect, got):
    import time
    t0 = time.time()
    while len(got) < expect:
        got += server.poll()
        assert time.time() - t0 < 120, "frames did not finish"
    return got


def _state(server, sid, cfg):
    import torch
    from volumefusion_gb300.fusion import FusionSession
    s = FusionSession.attach(server.session_handle(sid), cfg)
    torch.cuda.synchronize()
    t, w = s.tsdf()
    _, _, T = s.graph()
    return t.cpu().numpy(), w.cpu().numpy(), T.cpu().numpy()


@pytest.mark.gpu
def test_session_results_same_alone_and_in_a_mix():
    from volumefusion_gb300.serve import Server
    mix = _mix_configs()
    cfg_a, frames_a = mix[0]
    # alone
    srv = Server(8 << 30)
    sid = srv.open(cfg_a)
    res = []
    for i, mm in enumerate(frames_a):
        while not srv.submit(sid, mm, tag=i):
            res += srv.poll()
    res = _drain(srv, len(frames_a), res)
    alone = _state(srv, sid, cfg_a)
    assert [r[1] for r in res] == list(range(len(frames_a)))
    assert all(r[3]["error"] == 0 for r in res)
    srv.close()
    # in a mix: three sessions, frames submitted round-robin without waiting
    srv = Server(8 << 30)
    sids = [srv.open(cfg) for cfg, _ in mix]
    assert None not in sids
    total, res = 0, []
    for i in range(len(frames_a)):
        for sid_k, (cfg, frames) in zip(sids, mix):
            while not srv.submit(sid_k, frames[i], tag=i):
                res += srv.poll()
            total += 1
    res = _drain(srv, total, res)
    for sid_k in sids:
        tags = [r[1] for r in res if r[0] == sid_k]
        assert tags == list(range(len(frames_a)))
    assert all(r[3]["error"] == 0 for r in res)
    mixed = _state(srv, sids[0], cfg_a)
    for x, y in zip(alone, mixed):
        assert np.array_equal(x, y)
    usage = srv.usage()
    assert usage["sessions"] == 3
    for sid_k in sids:
        srv.close_session(sid_k)
    srv.poll()
    assert srv.usage()["sessions"] == 0 and srv.usage()["used_bytes"] == 0
    srv.close()


def test_admission_follows_the_memory_budget():
    """A session whose bytes do not fit the budget is refused before anything is allocated."""
    from volumefusion_gb300 import configs
    from volumefusion_gb300.serve import Server, session_bytes
    cfg = configs.small_nonrigid()
    need = session_bytes(cfg)
    assert need > 0
    srv = Server(need - 1)
    assert srv.open(cfg) is None
    u = srv.usage()
    assert u["sessions"] == 0 and u["denied"] == 1 and u["used_bytes"] == 0
    srv.close()


@pytest.mark.gpu
def test_closed_session_is_reused_with_fresh_results():
    """A closed session is reset and handed out again to an open with equal parameters (arena,
    stream and captured frame graphs kept); the frames it then fuses give exactly the state a
    fresh session gives.  An open with other parameters does not take it, and one that needs its
    memory evicts it."""
    from volumefusion_gb300.serve import Server, session_bytes
    mix = _mix_configs()
    cfg_a, frames_a = mix[0]
    cfg_c, frames_c = mix[2]
    srv = Server(8 << 30)

    def run(sid, frames):
        res = []
        for i, mm in enumerate(frames):
            while not srv.submit(sid, mm, tag=i):
                res += srv.poll()
        res = _drain(srv, len(frames), res)
        assert [r[1] for r in res] == list(range(len(frames)))
        assert all(r[3]["error"] == 0 for r in res)

    sid = srv.open(cfg_a)
    run(sid, frames_a)
    fresh = _state(srv, sid, cfg_a)
    srv.close_session(sid)
    srv.poll()
    c = srv.counters()
    assert c["opens_fresh"] == 1 and c["idle_sessions"] == 1 and srv.usage()["used_bytes"] == 0
    sid_c = srv.open(cfg_c)  # other parameters: a new session
    assert srv.counters()["opens_fresh"] == 2 and srv.counters()["idle_sessions"] == 1
    sid2 = srv.open(cfg_a)  # the idle one, reset
    c = srv.counters()
    assert c["opens_reused"] == 1 and c["idle_sessions"] == 0
    run(sid2, frames_a)
    again = _state(srv, sid2, cfg_a)
    for x, y in zip(fresh, again):
        assert np.array_equal(x, y)
    run(sid_c, frames_c)
    srv.close()
    # a budget that holds one session at a time: the idle session makes room for the next
    need = max(session_bytes(cfg_a), session_bytes(cfg_c))
    srv = Server(need + need // 2)
    sid = srv.open(cfg_a)
    srv.close_session(sid)
    assert srv.counters()["idle_sessions"] == 1
    sid = srv.open(cfg_c)
    assert sid is not None
    c = srv.counters()
    assert c["evictions"] == 1 and c["idle_sessions"] == 0 and c["opens_fresh"] == 2
    srv.close()

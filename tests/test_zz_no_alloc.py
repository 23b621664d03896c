"""kamino_projection_noalloc: the projection for callers that cannot allocate
device memory (their device memory comes from a host framework's pool or is
fixed at start-up).  Its temporaries live in a fixed array inside the library,
so it must give the same fields as the handle-based projection stage, which
uses memory the handle allocated.  Calls in a row with different inputs check
that the shared array carries nothing from one call into the next: repeated
calls of one size (the tables the array already holds are reused, the
spectrum and solutions of the previous call are overwritten), a change of
size (the tables are reloaded) and a return to the first size.

This file is named so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5  # relative L2, the step tests' tolerance


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _handle_projection(kg, st, nt):
    cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.005, fp64_modes=4)
    with kg.KaminoSolver(config=cfg) as s:
        s.load(st)
        s.projection()
        return s.fields()


def _noalloc(kg, torch, st, nt, alias):
    dev = torch.device("cuda")
    u = torch.from_numpy(st["u_phi"]).to(dev)
    v = torch.from_numpy(st["u_theta"]).to(dev)
    uo = u if alias else torch.empty_like(u)
    vo = v if alias else torch.empty_like(v)
    po = torch.empty((nt, 2 * nt), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()
    rc = kg.lib.kamino_projection_noalloc(nt, u.data_ptr(), v.data_ptr(), uo.data_ptr(), vo.data_ptr(),
                                          po.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, kg._lib.last_error()
    torch.cuda.synchronize()
    return {"u_phi": uo.cpu().numpy(), "u_theta": vo.cpu().numpy(), "pressure": po.cpu().numpy()}


def test_projection_noalloc_matches_handle_projection(kg, orc):
    torch = _torch()
    for call, (nt, seed) in enumerate([(128, 11), (128, 13), (256, 12), (128, 14)]):
        st = kg.make_initial_state(nt, lmax=8, seed=seed)
        want = _handle_projection(kg, st, nt)
        got = _noalloc(kg, torch, st, nt, alias=False)
        for k in got:
            err = orc.rel_l2(got[k], want[k])
            assert err <= TOL, "call %d (nt=%d) %s: rel L2 %.3e" % (call, nt, k, err)


def test_projection_noalloc_outputs_may_alias_inputs(kg, orc):
    """The header allows u_phi_out == u_phi and u_theta_out == u_theta: each
    value is read once, before the one write of the same place."""
    torch = _torch()
    for nt, seed in ((64, 21), (256, 22)):
        st = kg.make_initial_state(nt, lmax=8, seed=seed)
        want = _noalloc(kg, torch, st, nt, alias=False)
        got = _noalloc(kg, torch, st, nt, alias=True)
        for k in got:
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), (nt, k)


def test_projection_noalloc_rejects_sizes_beyond_the_limit(kg):
    torch = _torch()
    x = torch.zeros(8, device="cuda")
    for nt in (512, 48, 16):
        rc = kg.lib.kamino_projection_noalloc(nt, x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                                              x.data_ptr(), None)
        assert rc == kg.ERR_INVALID
        assert "n_theta" in kg._lib.last_error()

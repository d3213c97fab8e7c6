"""g6_force_noalloc: the allocation-free force entry point, checked against
g6_force (the context entry point) on two calls in a row.

Some callers cannot call cudaMalloc -- their device memory belongs to their
own arena or pool -- so this entry point takes device buffers from the caller
and keeps its intermediate tables in a static device array.  This file is
collected last so that a failure here cannot stop the other tests.
"""
import ctypes

import numpy as np
import pytest

import genesis6_gb300 as g6
from genesis6_gb300 import _capi, config

pytestmark = pytest.mark.gpu


def _noalloc(torch, model, path, b, rc, prec=_capi.FP64):
    L = g6.lib()
    n = len(b["com"])
    dev = torch.device("cuda")
    com = torch.tensor(b["com"], dtype=torch.float64, device=dev).contiguous()
    quat = torch.tensor(b["quat"], dtype=torch.float64, device=dev).contiguous()
    F = torch.full((n, 3), np.nan, dtype=torch.float64, device=dev)
    tau = torch.full((n, 3), np.nan, dtype=torch.float64, device=dev)
    ep = torch.full((1,), np.nan, dtype=torch.float64, device=dev)
    box = np.ascontiguousarray(b["L"], dtype=np.float64)
    st = L.g6_force_noalloc(_capi.MODELS[model], _capi.PATHS[path], prec, n, _capi.dptr(box), rc - 2.0, rc,
                            1.0, ctypes.c_void_p(com.data_ptr()), ctypes.c_void_p(quat.data_ptr()),
                            ctypes.c_void_p(F.data_ptr()), ctypes.c_void_p(tau.data_ptr()),
                            ctypes.c_void_p(ep.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == _capi.G6_OK
    return F.cpu().numpy(), tau.cpu().numpy(), float(ep.cpu().numpy()[0])


def _reference(model, path, b, rc):
    s = g6.RigidWater(model, len(b["com"]), b["L"], path=path, precision="fp64", rc=rc)
    s.upload_poses(b["com"], b["quat"])
    F, tau, ep, _ = s.force()
    s.close()
    return F, tau, ep[0]


def test_noalloc_matches_force_entry_twice():
    torch = pytest.importorskip("torch")
    cases = [("TIP4P", "custom", config.water_box("TIP4P", 4096, 77, jitter=0.4), 9.0),
             ("ST2", "custom", config.water_box("ST2", 1000, 78, jitter=0.4), 8.5)]
    for model, path, b, rc in cases:   # two calls in a row, different systems
        F, tau, ep = _noalloc(torch, model, path, b, rc)
        Fr, tr, er = _reference(model, path, b, rc)
        frms = np.sqrt((Fr ** 2).sum(1).mean()); trms = np.sqrt((tr ** 2).sum(1).mean())
        assert ep == pytest.approx(er, rel=1e-12)
        assert np.abs(F - Fr).max() <= 1e-12 * frms
        assert np.abs(tau - tr).max() <= 1e-12 * trms


def test_noalloc_mixed_and_std_paths():
    """The mixed-precision list kernel and the StdForce path through the
    no-alloc argument blocks: mixed against the FP64 context result at the
    mixed-precision bar (relative RMS force/torque error <= 1e-5), the std
    path in FP64 against the context at 1e-12; two calls in a row each."""
    torch = pytest.importorskip("torch")
    b4 = config.water_box("TIP4P", 2048, 91, jitter=0.4)
    b5 = config.water_box("TIP5P", 1000, 92, jitter=0.4)
    for model, path, b, rc in (("TIP4P", "custom", b4, 9.0), ("TIP5P", "std", b5, 8.5)):
        Fr, tr, er = _reference(model, path, b, rc)
        for _ in range(2):
            F, tau, ep = _noalloc(torch, model, path, b, rc, prec=_capi.MIXED)
            ef = np.sqrt(((F - Fr) ** 2).sum() / (Fr ** 2).sum())
            et = np.sqrt(((tau - tr) ** 2).sum() / (tr ** 2).sum())
            assert ef <= 1e-5 and et <= 1e-5, (model, ef, et)
            assert ep == pytest.approx(er, rel=1e-5)
    for _ in range(2):
        F, tau, ep = _noalloc(torch, "TIP5P", "std", b5, 8.5)
        Fr, tr, er = _reference("TIP5P", "std", b5, 8.5)
        frms = np.sqrt((Fr ** 2).sum(1).mean()); trms = np.sqrt((tr ** 2).sum(1).mean())
        assert ep == pytest.approx(er, rel=1e-12)
        assert np.abs(F - Fr).max() <= 1e-12 * frms
        assert np.abs(tau - tr).max() <= 1e-12 * trms


def test_noalloc_rejects_bad_cutoffs():
    """A negative r_in, r_in >= r_out and r_out above half the box are refused
    on the host before any device work (the buffers are real and sized)."""
    torch = pytest.importorskip("torch")
    L = g6.lib()
    n = 100
    box = np.array([30.0, 30.0, 30.0])
    buf = [torch.zeros(n * k, dtype=torch.float64, device="cuda") for k in (3, 4, 3, 3, 1)]
    ptrs = [ctypes.c_void_p(t.data_ptr()) for t in buf]
    for r_in, r_out in ((-1.0, 9.0), (9.0, 9.0), (7.0, 16.0)):
        st = L.g6_force_noalloc(_capi.TIP4P, _capi.PATH_CUSTOM, _capi.FP64, n, _capi.dptr(box), r_in, r_out, 1.0,
                                *ptrs, None)
        assert st == _capi.G6_ERR_ARG


def test_noalloc_rejects_oversized_system():
    L = g6.lib()
    box = np.array([100.0, 100.0, 100.0])
    st = L.g6_force_noalloc(_capi.TIP4P, _capi.PATH_CUSTOM, _capi.FP64, 5000,
                            _capi.dptr(box), 7.0, 9.0, 1.0, None, None, None, None, None, None)
    assert st == _capi.G6_ERR_CAPACITY

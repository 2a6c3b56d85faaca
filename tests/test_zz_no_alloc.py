"""The allocation-free entry point, gb_fwi2d_batch_noalloc, against gb_fwi2d_batch.

Some callers cannot allocate device memory while they run: their device
memory belongs to another runtime or to a fixed pool, an allocation would
stall a latency-critical loop, or a plain C caller has no way to hand over a
workspace.  gb_fwi2d_batch_noalloc serves them from a fixed scratch array the
library reserves on each GPU.  These tests call it through the C ABI twice in
a row and check both results against the ordinary entry point with a caller
workspace, at the tolerances of the other parity tests: synthetic data bit
for bit, gradient relative L2 <= 1e-4, misfit relative <= 1e-5.  The cases
cover one resident wave, 36 solves in several waves called from a fresh
host thread (the ordinary entry point would run them on two streams; this one
must create no stream), forward-only runs, synthetic data kept in the scratch (syn = NULL) and a
checkpointed 120 x 250, nt 2000 gradient batch, whose stored field would
never fit the scratch.

The file is named to be collected last, so a run that stops at the first
failure has run every other test before this one.
"""
import ctypes
import os
import threading

import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(cases.__file__)


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def run_both(lib, p, vels, obs_np, flags, keep_syn=True, calls=2, in_thread=False):
    """gb_fwi2d_batch once, then gb_fwi2d_batch_noalloc `calls` times; compare.
    Returns how many side streams the library created during the noalloc calls."""
    from geopvi_gb300 import _native
    dev = torch.device("cuda:0")
    n = vels.shape[0]
    vel = torch.from_numpy(np.ascontiguousarray(vels, dtype=np.float32)).to(dev)
    obs = torch.from_numpy(np.ascontiguousarray(obs_np, dtype=np.float32)).to(dev)
    cp = p.c()
    fwd = bool(flags & _native.FLAG_FORWARD_ONLY)

    def outputs():
        syn = torch.empty(n, p.data_len, dtype=torch.float32, device=dev) if keep_syn else None
        grad = None if fwd else torch.empty(n, p.ncell, dtype=torch.float32, device=dev)
        return syn, grad, torch.empty(n, dtype=torch.float64, device=dev)

    def ptr(t):
        return None if t is None else t.data_ptr()

    stream = torch.cuda.current_stream(dev).cuda_stream
    base_flags = flags & ~_native.FLAG_CHECKPOINT  # reference run: full storage
    nbytes = lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), n, 0, base_flags)
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    syn0, grad0, mis0 = outputs()
    st = lib.gb_fwi2d_batch(ctypes.byref(cp), n, vel.data_ptr(), obs.data_ptr(), ptr(syn0), ptr(grad0),
                            mis0.data_ptr(), base_flags, 0, work.data_ptr(), nbytes, stream)
    assert st == 0
    torch.cuda.synchronize(dev)
    del work

    results = []

    def noalloc_calls():
        for call in range(calls):  # the scratch keeps the previous call's contents
            syn1, grad1, mis1 = outputs()
            st = lib.gb_fwi2d_batch_noalloc(ctypes.byref(cp), n, vel.data_ptr(), obs.data_ptr(), ptr(syn1),
                                            ptr(grad1), mis1.data_ptr(), flags, stream)
            torch.cuda.synchronize(dev)
            results.append((st, lib.gb_fwi2d_status(None, stream), syn1, grad1, mis1))

    streams_before = lib.gb_fwi2d_side_stream_count()
    if in_thread:  # a host thread that has made no CUDA call yet and holds no side stream
        t = threading.Thread(target=noalloc_calls)
        t.start()
        t.join()
    else:
        noalloc_calls()
    new_streams = lib.gb_fwi2d_side_stream_count() - streams_before
    assert len(results) == calls
    for call, (st, status, syn1, grad1, mis1) in enumerate(results):
        assert st == 0, f"call {call}: status {st}"
        assert status == 0, f"call {call}: device status {status}"
        if keep_syn:
            assert torch.equal(syn1, syn0), f"call {call}: synthetic data differ"
        if not fwd:
            assert rel(grad1.cpu().numpy(), grad0.cpu().numpy()) <= 1e-4, f"call {call}"
        m0, m1 = mis0.cpu().numpy(), mis1.cpu().numpy()
        assert np.all(np.abs(m1 - m0) <= 1e-5 * np.abs(m0)), f"call {call}"
    return new_streams


def golden(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    return z, cases.params_from_npz(z)


@pytest.mark.parametrize("name", ["fwi_o8_nti2", "img_o6"])
def test_noalloc_matches_workspace_entry_point(engine_lib, cuda, name):
    from geopvi_gb300 import _native
    z, p = golden(name)
    flags = 0 if int(z["run_fwi"]) else _native.FLAG_IMAGING
    vels = np.stack([z["start"], z["truth"], z["start"] * np.float32(1.02)])
    run_both(engine_lib, p, vels, z["obs"], flags)


def test_noalloc_many_resident_solves_one_stream(engine_lib, cuda):
    """fwi_o8 x 12 samples = 36 solves: more than 32 resident at once and, in 64 MiB,
    more than one wave, called from a host thread that has made no CUDA call yet.  The
    ordinary entry point runs such waves on two streams; this one must create none."""
    z, p = golden("fwi_o8")
    rng = np.random.default_rng(5)
    vels = np.stack([z["start"] * np.float32(1.0 + 0.01 * rng.standard_normal()) for _ in range(12)])
    assert run_both(engine_lib, p, vels, z["obs"], 0, in_thread=True) == 0


@pytest.mark.parametrize("flags_name", ["forward_only", "syn_in_scratch"])
def test_noalloc_forward_only_and_scratch_data(engine_lib, cuda, flags_name):
    from geopvi_gb300 import _native
    z, p = golden("fwi_o8")
    vels = np.stack([z["start"], z["truth"]])
    if flags_name == "forward_only":
        run_both(engine_lib, p, vels, z["obs"], _native.FLAG_FORWARD_ONLY)
    else:
        run_both(engine_lib, p, vels, z["obs"], 0, keep_syn=False)


def test_noalloc_checkpointed_full_size_gradient(engine_lib, cuda):
    """One 120 x 250, nt 2000, 10-shot gradient batch: full storage needs ~2.5 GB, the
    checkpointed scratch run holds two solves at a time in 64 MiB."""
    from geopvi_gb300 import _native, workloads
    w = workloads.cfg1(nsamples=1)
    p = w.params
    dev = torch.device("cuda:0")
    cp = p.c()
    stream = torch.cuda.current_stream(dev).cuda_stream
    truth = torch.from_numpy(w.truth).to(dev).unsqueeze(0)
    zeros = torch.zeros(p.data_len, dtype=torch.float32, device=dev)
    obs = torch.empty(1, p.data_len, dtype=torch.float32, device=dev)
    nbytes = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 1, 0, _native.FLAG_FORWARD_ONLY)
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(cp), 1, truth.data_ptr(), zeros.data_ptr(), obs.data_ptr(), None,
                                   None, _native.FLAG_FORWARD_ONLY, 0, work.data_ptr(), nbytes, stream)
    assert st == 0
    torch.cuda.synchronize(dev)
    del work
    run_both(engine_lib, p, w.samples[:1], obs.cpu().numpy()[0], _native.FLAG_CHECKPOINT)


def test_noalloc_rejects_batches_beyond_the_scratch(engine_lib, cuda):
    from geopvi_gb300 import _native
    from geopvi_gb300.params import Params
    # 2000 x 2000 interior: the padded v*dt of one sample alone exceeds the scratch
    p = Params(nx=2000, nz=2000, pml0=20, Lc=4, ns=64, nt=4000, ds=30, ns0=10, depths=2, depthr=0,
               nr=2000, dr=1, nr0=0, nt_interval=1, dx=10.0, dz=10.0, dt=1e-3, f0=10.0)
    cp = p.c()
    dev = torch.device("cuda:0")
    dummy = torch.zeros(16, dtype=torch.float32, device=dev)
    st = engine_lib.gb_fwi2d_batch_noalloc(ctypes.byref(cp), 4, dummy.data_ptr(), dummy.data_ptr(), None, None,
                                           None, 0, torch.cuda.current_stream(dev).cuda_stream)
    assert st == _native.E2BIG

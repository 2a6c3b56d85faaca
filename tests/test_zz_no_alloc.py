"""The allocation-free entry point, gb_fwi2d_batch_noalloc, against gb_fwi2d_batch.

Some callers cannot allocate device memory while they run (their device
memory belongs to another runtime or to a fixed pool, or an allocation would
stall a latency-critical loop).  gb_fwi2d_batch_noalloc serves them from a
fixed scratch array the library reserves on each GPU.  This test calls it
through the C ABI twice in a row and checks both results against the
ordinary entry point with a caller workspace, at the tolerances of the other
parity tests: synthetic data bit for bit, gradient relative L2 <= 1e-4,
misfit relative <= 1e-5.

The file is named to be collected last, so a run that stops at the first
failure has run every other test before this one.
"""
import ctypes
import os

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


@pytest.mark.parametrize("name", ["fwi_o8_nti2", "img_o6"])
def test_noalloc_matches_workspace_entry_point(engine_lib, cuda, name):
    from geopvi_gb300 import _native
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = cases.params_from_npz(z)
    flags = 0 if int(z["run_fwi"]) else _native.FLAG_IMAGING
    vels = np.stack([z["start"], z["truth"], z["start"] * np.float32(1.02)]).astype(np.float32)
    n = vels.shape[0]
    dev = torch.device("cuda:0")
    vel = torch.from_numpy(vels).to(dev)
    obs = torch.from_numpy(np.ascontiguousarray(z["obs"], dtype=np.float32)).to(dev)
    cp = p.c()
    stream = torch.cuda.current_stream(dev).cuda_stream

    def outputs():
        return (torch.empty(n, p.data_len, dtype=torch.float32, device=dev),
                torch.empty(n, p.ncell, dtype=torch.float32, device=dev),
                torch.empty(n, dtype=torch.float64, device=dev))

    # ordinary entry point, caller-provided workspace
    nbytes = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), n, 0, flags)
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    syn0, grad0, mis0 = outputs()
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(cp), n, vel.data_ptr(), obs.data_ptr(), syn0.data_ptr(),
                                   grad0.data_ptr(), mis0.data_ptr(), flags, 0, work.data_ptr(), nbytes, stream)
    assert st == 0
    torch.cuda.synchronize(dev)

    for call in range(2):  # the scratch keeps the previous call's contents
        syn1, grad1, mis1 = outputs()
        st = engine_lib.gb_fwi2d_batch_noalloc(ctypes.byref(cp), n, vel.data_ptr(), obs.data_ptr(),
                                               syn1.data_ptr(), grad1.data_ptr(), mis1.data_ptr(), flags, stream)
        assert st == 0, f"call {call}: status {st}"
        torch.cuda.synchronize(dev)
        assert torch.equal(syn1, syn0), f"call {call}: synthetic data differ"
        assert rel(grad1.cpu().numpy(), grad0.cpu().numpy()) <= 1e-4, f"call {call}"
        m0, m1 = mis0.cpu().numpy(), mis1.cpu().numpy()
        assert np.all(np.abs(m1 - m0) <= 1e-5 * np.abs(m0)), f"call {call}"


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

"""gb_fwi2d_run_instances: an uneven batch (per-instance parameter sets) on one stream.

Host side (no GPU): the workspace query is the largest instance's, and every
instance is checked before anything is enqueued.  On the GPU: each
instance's outputs equal the same instance run alone through gb_fwi2d_batch,
bit for bit (the data) and within the gradient's FP32 reduction order (the
same kernels, so also bit for bit here).
"""
import ctypes
import os

import numpy as np
import pytest

import cases
from geopvi_gb300 import _native

GOLDEN = os.path.dirname(cases.__file__)


def params(name):
    return cases.params_from_npz(np.load(os.path.join(GOLDEN, name + ".npz")))


def instance(p, nsamples=1, vel=1, obs=1, syn=None, grad=1, misfit=None):
    return _native.CInstance(p.c(), nsamples, vel, obs, syn, grad, misfit)


def test_workspace_is_the_largest_instances(engine_lib):
    ps = [params(n) for n in ("fwi_o8", "fwi_o12", "fwi_ragged")]
    arr = (_native.CInstance * 3)(*[instance(p, nsamples=k + 1) for k, p in enumerate(ps)])
    sizes = [engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), k + 1, 0, 0) for k, p in enumerate(ps)]
    assert engine_lib.gb_fwi2d_instances_workspace_bytes(arr, 3, 0, 0) == max(sizes)
    bad = (_native.CInstance * 2)(instance(ps[0]), instance(ps[1], nsamples=0))
    assert engine_lib.gb_fwi2d_instances_workspace_bytes(bad, 2, 0, 0) == 0


def test_everything_checked_before_anything_runs(engine_lib):
    """Invalid entries anywhere in the array fail up front (no device call is
    made, so this runs without a GPU)."""
    ps = [params("fwi_o8"), params("fwi_o12")]
    big = 1 << 40
    ok = instance(ps[0])
    for badinst in (instance(ps[1], nsamples=0), instance(ps[1], vel=None), instance(ps[1], grad=None)):
        arr = (_native.CInstance * 2)(ok, badinst)
        assert engine_lib.gb_fwi2d_run_instances(arr, 2, 0, 0, 1, big, None) == _native.EINVAL
    q = params("fwi_o12").replace(nx=0)
    arr = (_native.CInstance * 2)(ok, instance(q))
    assert engine_lib.gb_fwi2d_run_instances(arr, 2, 0, 0, 1, big, None) == _native.EINVAL
    arr = (_native.CInstance * 2)(ok, instance(ps[1], nsamples=4))
    need = engine_lib.gb_fwi2d_instances_workspace_bytes(arr, 2, 0, 0)
    assert engine_lib.gb_fwi2d_run_instances(arr, 2, 0, 0, 1, need - 1, None) == _native.ENOMEM
    arr = (_native.CInstance * 1)(ok)
    assert engine_lib.gb_fwi2d_run_instances(arr, 1, _native.FLAG_EXACT_GRADIENT | _native.FLAG_IMAGING, 0, 1,
                                             big, None) == _native.EINVAL
    assert engine_lib.gb_fwi2d_run_instances(arr, 0, 0, 0, 1, big, None) == _native.EINVAL


@pytest.mark.gpu
def test_uneven_instances_match_single_batches(engine_lib, cuda):
    import torch
    names = ("fwi_o8", "fwi_o12", "fwi_ragged")
    stream = torch.cuda.current_stream(cuda).cuda_stream
    insts, keep, alone = [], [], []
    for k, name in enumerate(names):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        p = cases.params_from_npz(z)
        n = k + 1
        vels = np.stack([z["start"] * np.float32(1 + 0.01 * i) for i in range(n)]).astype(np.float32)
        vel = torch.from_numpy(vels).to(cuda)
        obs = torch.from_numpy(np.ascontiguousarray(z["obs"], dtype=np.float32)).to(cuda)
        out = (torch.empty(n, p.data_len, device=cuda), torch.empty(n, p.ncell, device=cuda),
               torch.empty(n, dtype=torch.float64, device=cuda))
        insts.append(_native.CInstance(p.c(), n, vel.data_ptr(), obs.data_ptr(), out[0].data_ptr(),
                                       out[1].data_ptr(), out[2].data_ptr()))
        keep.append((vel, obs, out))
        nb = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), n, 0, 0)
        work = torch.empty(nb, dtype=torch.uint8, device=cuda)
        ref = (torch.empty(n, p.data_len, device=cuda), torch.empty(n, p.ncell, device=cuda),
               torch.empty(n, dtype=torch.float64, device=cuda))
        assert engine_lib.gb_fwi2d_batch(ctypes.byref(p.c()), n, vel.data_ptr(), obs.data_ptr(), ref[0].data_ptr(),
                                         ref[1].data_ptr(), ref[2].data_ptr(), 0, 0, work.data_ptr(), nb,
                                         stream) == 0
        alone.append(ref)
    arr = (_native.CInstance * len(insts))(*insts)
    nbytes = engine_lib.gb_fwi2d_instances_workspace_bytes(arr, len(insts), 0, 0)
    work = torch.empty(nbytes, dtype=torch.uint8, device=cuda)
    assert engine_lib.gb_fwi2d_run_instances(arr, len(insts), 0, 0, work.data_ptr(), nbytes, stream) == 0
    torch.cuda.synchronize(cuda)
    assert engine_lib.gb_fwi2d_last_launch_count() > 0
    for (_, _, out), ref in zip(keep, alone):
        for a, b in zip(out, ref):
            assert torch.equal(a, b)

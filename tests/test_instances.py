"""gb_fwi2d_run_instances: an uneven batch (per-instance parameter sets) on one stream.

Host side (no GPU): the workspace query is the largest instance's, and every
instance is checked before anything is enqueued.  On the GPU: each
instance's outputs equal the same instance run alone through gb_fwi2d_batch,
bit for bit -- the fused launches (solves of several instances in one wave,
an instance's solves split over waves, pieces ending at different steps) run
every solve through the same tile code with its own buffers.
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


def test_workspace_query(engine_lib):
    """Unfused (here: checkpointed) instances run one after another in the
    workspace of the largest; fused ones need the largest's kept buffers and
    one resident solve, and waves fill whatever more the caller gives."""
    ps = [params(n) for n in ("fwi_o8", "fwi_o12", "fwi_ragged")]
    arr = (_native.CInstance * 3)(*[instance(p, nsamples=k + 1) for k, p in enumerate(ps)])
    ws = lambda p, n, r, f: engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), n, r, f)  # noqa: E731
    ck = _native.FLAG_CHECKPOINT
    assert engine_lib.gb_fwi2d_instances_workspace_bytes(arr, 3, 0, ck) == max(
        ws(p, k + 1, 0, ck) for k, p in enumerate(ps))
    fused = engine_lib.gb_fwi2d_instances_workspace_bytes(arr, 3, 0, 0)
    assert max(ws(p, k + 1, 1, 0) for k, p in enumerate(ps)) <= fused < max(ws(p, k + 1, 0, 0) for k, p in
                                                                            enumerate(ps))
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


FUSED = ("fwi_o8", "fwi_ragged", "fwi_o8_nti2", "fwi_nr1", "fwi_pml1", "fwi_o12", "fwi_o10_nti3", "img_o6")


def _fused_setup(cuda, names, flags, syn_none=()):
    import torch
    stream = torch.cuda.current_stream(cuda).cuda_stream
    insts, keep, alone, nts = [], [], [], {}
    fwd_only = bool(flags & _native.FLAG_FORWARD_ONLY)
    for k, name in enumerate(names):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        p = cases.params_from_npz(z)
        n = 1 + k % 3
        vels = np.stack([z["start"] * np.float32(1 + 0.01 * i) for i in range(n)]).astype(np.float32)
        vel = torch.from_numpy(vels).to(cuda)
        obs = torch.from_numpy(np.ascontiguousarray(z["obs"], dtype=np.float32)).to(cuda)
        own_syn = name not in syn_none

        def outs():
            return (torch.full((n, p.data_len), -1.0, device=cuda) if own_syn else None,
                    None if fwd_only else torch.full((n, p.ncell), -1.0, device=cuda),
                    torch.full((n,), -1.0, dtype=torch.float64, device=cuda))
        out, ref = outs(), outs()
        ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
        insts.append(_native.CInstance(p.c(), n, vel.data_ptr(), obs.data_ptr(), ptr(out[0]), ptr(out[1]),
                                       ptr(out[2])))
        keep.append((vel, obs, out))
        alone.append((p, n, vel, obs, ref))
        nts[name] = ((p.Lc, p.nz, p.nx, p.pml0, p.dx, p.dz, p.dt), p.nt)
    return stream, insts, keep, alone, nts


def _run_alone(engine_lib, cuda, alone, flags, stream):
    import torch
    for p, n, vel, obs, ref in alone:
        nb = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), n, 0, flags)
        work = torch.empty(nb, dtype=torch.uint8, device=cuda)
        ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
        assert engine_lib.gb_fwi2d_batch(ctypes.byref(p.c()), n, vel.data_ptr(), obs.data_ptr(), ptr(ref[0]),
                                         ptr(ref[1]), ptr(ref[2]), flags, 0, work.data_ptr(), nb, stream) == 0
        torch.cuda.synchronize(cuda)


@pytest.mark.gpu
@pytest.mark.parametrize("room,max_resident,flags", [
    ("min", 0, 0),                              # the query's size: waves, instances split over them
    ("all", 0, 0),                              # room for everything: one wave per FD order
    ("all", 3, 0),                              # at most 3 solves per wave: many pieces
    ("all", 0, _native.FLAG_IMAGING),
    ("all", 0, _native.FLAG_FORWARD_ONLY),
])
def test_fused_waves_match_single_batches(engine_lib, cuda, room, max_resident, flags):
    import torch
    stream, insts, keep, alone, nts = _fused_setup(cuda, FUSED, flags, syn_none=("fwi_nr1", "img_o6"))
    _run_alone(engine_lib, cuda, alone, flags, stream)
    arr = (_native.CInstance * len(insts))(*insts)
    nbytes = engine_lib.gb_fwi2d_instances_workspace_bytes(arr, len(insts), max_resident, flags)
    if room == "all":
        nbytes = sum(engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), n, 0, flags)
                     for p, n, *_ in alone) + (8 << 20)
    work = torch.full((nbytes,), 0xFF, dtype=torch.uint8, device=cuda)
    assert engine_lib.gb_fwi2d_run_instances(arr, len(insts), flags, max_resident, work.data_ptr(), nbytes,
                                             stream) == 0
    torch.cuda.synchronize(cuda)
    assert engine_lib.gb_fwi2d_status(ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(stream)) == 0
    for (_, _, out), (*_, ref) in zip(keep, alone):
        for a, b in zip(out, ref):
            if a is not None:
                assert torch.equal(a, b)
    if room == "all" and max_resident == 0:
        # one wave per FD order: per instance k_prepare, the reduction and the
        # misfit's two kernels; per grid one launch per step and pass while
        # one of its instances runs
        fwd_only = bool(flags & _native.FLAG_FORWARD_ONLY)
        by_grid = {}
        for key, nt in nts.values():
            by_grid[key] = max(by_grid.get(key, 0), nt)
        expect = len(insts) * (1 + (0 if fwd_only else 1) + 2) + sum(by_grid.values()) * (1 if fwd_only else 2)
        assert engine_lib.gb_fwi2d_last_launch_count() == expect


def test_fused_wave_plan(engine_lib):
    """The host-side plan of the fused path (no GPU): every instance fits at
    the queried size, however small; room for everything gives one wave per
    FD order; a cap on resident solves splits the waves."""
    names = FUSED
    ps = [params(n) for n in names]
    arr = (_native.CInstance * len(ps))(*[instance(p, nsamples=1 + k % 3) for k, p in enumerate(ps)])
    need = engine_lib.gb_fwi2d_instances_workspace_bytes(arr, len(ps), 0, 0)
    waves = engine_lib.gb_fwi2d_instances_waves(arr, len(ps), 0, 0, need)
    assert waves >= len({p.Lc for p in ps})
    assert engine_lib.gb_fwi2d_instances_waves(arr, len(ps), 0, 0, need - 1) == _native.ENOMEM
    assert engine_lib.gb_fwi2d_instances_waves(arr, len(ps), 0, 0, 1 << 40) == len({p.Lc for p in ps})
    solves = {}
    for k, p in enumerate(ps):
        solves[p.Lc] = solves.get(p.Lc, 0) + (1 + k % 3) * p.ns
    assert engine_lib.gb_fwi2d_instances_waves(arr, len(ps), 0, 3, 1 << 40) == sum(-(-s // 3) for s in solves.values())
    assert engine_lib.gb_fwi2d_instances_waves(arr, len(ps), _native.FLAG_CHECKPOINT, 0, 1 << 40) == _native.EINVAL
    # the uneven batch of 48 instances in a 150 GB workspace: ~2.1 TB of stored fields
    from geopvi_gb300 import workloads
    big = [instance(p) for p in workloads.cfg4_instances()]
    arr = (_native.CInstance * len(big))(*big)
    assert 10 <= engine_lib.gb_fwi2d_instances_waves(arr, len(big), 0, 0, 150 << 30) <= 20


@pytest.mark.gpu
def test_fused_halves_on_two_streams(engine_lib, cuda):
    """Two instances of one grid with 51 solves in one wave: the launch runs
    as two halves on two streams, cutting the first instance's piece at solve
    25 -- results still those of each instance alone."""
    import torch
    names = ("fwi_o8", "fwi_o8_nti2")
    stream = torch.cuda.current_stream(cuda).cuda_stream
    insts, keep, alone = [], [], []
    for name, n in zip(names, (12, 5)):
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        p = cases.params_from_npz(z)
        vels = np.stack([z["start"] * np.float32(1 + 0.005 * i) for i in range(n)]).astype(np.float32)
        vel = torch.from_numpy(vels).to(cuda)
        obs = torch.from_numpy(np.ascontiguousarray(z["obs"], dtype=np.float32)).to(cuda)
        out = (torch.full((n, p.data_len), -1.0, device=cuda), torch.full((n, p.ncell), -1.0, device=cuda),
               torch.full((n,), -1.0, dtype=torch.float64, device=cuda))
        insts.append(_native.CInstance(p.c(), n, vel.data_ptr(), obs.data_ptr(), out[0].data_ptr(),
                                       out[1].data_ptr(), out[2].data_ptr()))
        keep.append((vel, obs, out))
        alone.append((p, n, vel, obs, tuple(torch.empty_like(t) for t in out)))
    _run_alone(engine_lib, cuda, alone, 0, stream)
    arr = (_native.CInstance * 2)(*insts)
    nbytes = sum(engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), n, 0, 0) for p, n, *_ in alone) + (8 << 20)
    assert engine_lib.gb_fwi2d_instances_waves(arr, 2, 0, 0, nbytes) == 1
    work = torch.empty(nbytes, dtype=torch.uint8, device=cuda)
    assert engine_lib.gb_fwi2d_run_instances(arr, 2, 0, 0, work.data_ptr(), nbytes, stream) == 0
    torch.cuda.synchronize(cuda)
    assert engine_lib.gb_fwi2d_status(ctypes.c_void_p(work.data_ptr()), ctypes.c_void_p(stream)) == 0
    for (_, _, out), (*_, ref) in zip(keep, alone):
        for a, b in zip(out, ref):
            assert torch.equal(a, b)
    # two launches per step while both halves run: fwi_o8's 300 steps, fwi_o8_nti2's 301
    assert engine_lib.gb_fwi2d_last_launch_count() == 2 * (1 + 1 + 2) + 2 * (300 + 301)

"""C ABI and host-side logic, no GPU needed.

The library loads without a device; only the host-side entry points
(parameter file, validation, workspace sizing) are called here.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import cases
from geopvi_gb300 import _native
from geopvi_gb300.params import prepare_fwi_parameters, read_paramfile, write_paramfile

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "geopvi_fwi2d.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"^\s*#.*$", "", text, flags=re.M)  # preprocessor lines
    return sorted(set(re.findall(r"\b([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text)))


def test_header_lists_every_export():
    assert set(declared_functions()) == set(_native.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(engine_lib):
    for name in declared_functions():
        assert hasattr(engine_lib, name), f"{name} not exported"
    assert b"sm_103a" in engine_lib.gb_fwi2d_version()


def test_read_params_matches_writer(engine_lib, tmp_path):
    for c in cases.SMALL.values():
        p = c["params"]
        path = str(tmp_path / "input_param.txt")
        write_paramfile(path, p)
        back = read_paramfile(path)
        for f in _native.INT_FIELDS:
            assert getattr(back, f) == getattr(p, f)
        for f in _native.FLOAT_FIELDS:
            assert np.float32(getattr(back, f)) == np.float32(getattr(p, f))


def test_prepare_fwi_parameters_layout(engine_lib, tmp_path):
    """The INI -> positional file of posterior.py:27-68, read back by the C reader."""
    import configparser
    cfg = configparser.ConfigParser()
    cfg.read_string("""[FWI]
nx = 250
nz = 110
layer_fixed = 10
vel_fixed = 1950
pml = 10
Lc = 3
laplace_slover = 0
ns = 12
nt = 2001
ds = 20
ns0 = 15
depths = 1
depthr = 9
nr = 250
dr = 1
nr0 = 0
nt_interval = 2
dx = 20.0
dz = 20.0
dt = 0.002
f0 = 10.0
""")
    path = str(tmp_path / "input_params.txt")
    prepare_fwi_parameters(path, cfg)
    lines = open(path).read().splitlines()
    assert len(lines) == 38 and lines[0] == "--grid points in x direction (nx)" and lines[1] == "250"
    assert lines[-2] == "--Dominant frequency (f0)" and lines[-1] == "10.0"
    p = read_paramfile(path)
    assert (p.nx, p.nz, p.pml0, p.Lc, p.ns, p.nt, p.nt_interval) == (250, 110, 10, 3, 12, 2001, 2)


def test_missing_paramfile(engine_lib, tmp_path):
    with pytest.raises(FileNotFoundError):
        read_paramfile(str(tmp_path / "nope.txt"))


def _status(engine_lib, p):
    cp = p.c()
    return engine_lib.gb_fwi2d_validate(ctypes.byref(cp))


def test_validation_codes(engine_lib):
    good = cases.SMALL["fwi_o8"]["params"]
    assert _status(engine_lib, good) == _native.OK
    assert _status(engine_lib, good.replace(laplace_solver=1)) == _native.OK      # pseudo-spectral
    assert _status(engine_lib, good.replace(laplace_solver=2)) == _native.EINVAL
    assert _status(engine_lib, good.replace(Lc=7)) == _native.EINVAL
    assert _status(engine_lib, good.replace(nx=0)) == _native.EINVAL
    assert _status(engine_lib, good.replace(dr=0)) == _native.EINVAL          # 36 receivers in one cell
    assert _status(engine_lib, good.replace(ns0=10_000)) == _native.EINVAL    # source off the grid
    assert _status(engine_lib, good.replace(nr=500)) == _native.EINVAL        # receivers off the grid
    assert _status(engine_lib, good.replace(depths=-100)) == _native.EINVAL
    assert _status(engine_lib, good.replace(nt_interval=0)) == _native.EINVAL
    assert _status(engine_lib, good.replace(dt=0.0)) == _native.EINVAL


def test_workspace_sizing(engine_lib):
    p = cases.SMALL["fwi_o8"]["params"]
    cp = p.c()
    one = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 2, 1, 0)
    two = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 2, 2, 0)
    allr = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 2, 0, 0)
    fwd = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 2, 0, _native.FLAG_FORWARD_ONLY)
    assert 0 < one < two <= allr
    assert fwd < allr
    # one more resident solve costs three padded fields plus the stored snapshots
    per = two - one
    assert per >= 4 * (3 * p.ntp + p.nt_save * p.ncell)
    bad = p.replace(nx=-1).c()
    assert engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(bad), 2, 0, 0) == 0


def test_batch_rejects_bad_arguments_without_gpu(engine_lib):
    p = cases.SMALL["fwi_o8"]["params"]
    cp = p.c()
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(cp), 0, None, None, None, None, None, 0, 0, None, 0, None)
    assert st == _native.EINVAL
    bad = p.replace(laplace_solver=2).c()
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(bad), 1, 1, 1, None, None, None, 0, 0, 1, 1 << 30, None)
    assert st == _native.EINVAL
    # pseudo-spectral mode: no exact adjoint (it transposes the FD stencil), no static scratch
    ps = p.replace(laplace_solver=1).c()
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(ps), 1, 1, 1, None, None, None, _native.FLAG_EXACT_GRADIENT, 0, 1,
                                   1 << 30, None)
    assert st == _native.ENOTSUP
    assert engine_lib.gb_fwi2d_batch_noalloc(ctypes.byref(ps), 1, 1, 1, None, None, None, 0, None) == _native.ENOTSUP


def test_pseudo_spectral_workspace(engine_lib):
    """laplace_solver = 1 adds one dense complex-double transform array per resident solve."""
    p = cases.SMALL["fwi_o8"]["params"].replace(laplace_solver=1)
    assert p.pml == p.pml0  # no stencil halo in this mode (fdtd2D_modelling.c:75-78)
    same_grid = p.replace(laplace_solver=0, pml0=p.pml0 - (p.Lc + 1))  # the FD mode on the same padded grid
    assert same_grid.ntp == p.ntp
    fd = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(same_grid.c()), 2, 3, 0)
    ps = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(p.c()), 2, 3, 0)
    assert ps - fd >= 16 * p.ntp * 3


def test_checkpoint_workspace_is_smaller(engine_lib):
    from geopvi_gb300 import workloads
    p = workloads.cfg3().params
    cp = p.c()
    full = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 1, 32, 0)
    ck = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 1, 32, _native.FLAG_CHECKPOINT)
    # 32 solves of 300x600, nt 4000: full storage ~93 GB, checkpoints ~5 GB
    assert ck * 10 < full


def test_batch_plan_prefers_checkpoints_when_memory_is_tight(engine_lib):
    from geopvi_gb300 import workloads
    from geopvi_gb300.scheduler import plan_batch
    p = workloads.cfg3().params  # 300x600, nt 4000, 32 shots: ~2.9 GB stored field per solve
    roomy = plan_batch(p, 16, 4 << 40)
    assert roomy is not None and not roomy.checkpoint and roomy.resident == 16 * 32
    # 8 GB holds one full-storage solve beside the synthetic data, ~19 checkpointed ones
    tight = plan_batch(p, 16, 8 << 30)
    assert tight is not None and tight.checkpoint and tight.nbytes <= 8 << 30 and tight.resident > 10
    assert plan_batch(p, 16, 1 << 20) is None


def test_arena_first_fit_and_merge():
    from geopvi_gb300.scheduler import Arena
    a = Arena(10 * 256)
    x = a.alloc(300)   # 2 granules
    y = a.alloc(256)
    z = a.alloc(1000)  # 4 granules
    assert (x, y, z) == (0, 512, 768) and a.largest() == 3 * 256
    assert a.alloc(4 * 256) is None
    a.release(y, 256)
    a.release(x, 300)
    assert a.largest() == 3 * 256 and a.alloc(3 * 256) == 0
    a.release(0, 3 * 256)
    a.release(z, 1000)
    assert a.free == [(0, 10 * 256)]


def test_exact_gradient_workspace_and_flags(engine_lib):
    from geopvi_gb300 import workloads
    p = workloads.cfg3().params  # nt 4000: all levels vs one ~64-step segment
    cp = p.c()
    full = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 1, 4, _native.FLAG_EXACT_GRADIENT)
    seg = engine_lib.gb_fwi2d_workspace_bytes(ctypes.byref(cp), 1, 4,
                                              _native.FLAG_EXACT_GRADIENT | _native.FLAG_CHECKPOINT)
    assert 0 < seg * 10 < full
    # every forward level of every resident solve is kept
    assert full >= 4 * 4 * p.nt * p.ntp
    small = cases.SMALL["fwi_o8"]["params"].c()
    st = engine_lib.gb_fwi2d_batch(ctypes.byref(small), 1, 1, 1, None, None, None,
                                   _native.FLAG_EXACT_GRADIENT | _native.FLAG_IMAGING, 0, 1, 1 << 30, None)
    assert st == _native.EINVAL


def test_step_cost_model_sees_strips_and_launch_latency():
    """Per padded cell, a small grid (mostly absorbing strips) costs more than a
    large one, and a one-solve step is dominated by the launch's fixed cost."""
    from geopvi_gb300 import workloads
    from geopvi_gb300.scheduler import LAUNCH_OVERHEAD_S, step_seconds
    small = workloads.make_params(100, 200, 1500, 1e-3, 4, 8.0)
    large = workloads.make_params(400, 800, 1500, 1e-3, 4, 8.0)
    per_cell = lambda p: (step_seconds(p, 1000) - LAUNCH_OVERHEAD_S) / (1000 * p.ntp)  # noqa: E731
    assert per_cell(small) > 1.2 * per_cell(large)
    assert step_seconds(small, 1) < 2 * LAUNCH_OVERHEAD_S


def test_server_merges_queued_requests_per_inversion():
    """The dispatcher's groups: one per inversion in queue order, requests of
    one inversion merged up to max_group_samples (built without a GPU)."""
    import numpy as np
    import torch
    from geopvi_gb300.scheduler import FwiServer, Request
    srv = FwiServer.__new__(FwiServer)
    srv.max_group_samples = 8
    srv._pending = [Request(n, torch.zeros(k, 4)) for n, k in
                    [("a", 3), ("b", 2), ("a", 4), ("a", 2), ("c", 9), ("b", 1)]]
    groups = srv._groups()
    assert [(name, [r.nsamples for r in reqs], n) for name, reqs, n in groups] == [
        ("a", [3, 4], 7), ("b", [2, 1], 3), ("c", [9], 9)]
    assert np.sum([n for *_, n in groups]) == 19


def test_fused_call_chosen_by_cost():
    """Many small instances (the uneven batch of 48) fuse; a few requests
    whose full storage is ~100x the workspace run their own, checkpointed
    plans instead (the fused call would run waves of a few solves)."""
    from geopvi_gb300 import workloads
    from geopvi_gb300.scheduler import fused_seconds, plan_batch
    cap = 150 << 30
    uneven = [(p, 1) for p in workloads.cfg4_instances()]
    alone = sum(plan_batch(p, n, cap).est_seconds for p, n in uneven)
    assert fused_seconds(uneven, cap) < 0.8 * alone
    big = [(workloads.make_params(400, 800, 5000, 1e-3, 40, 8.0), 32),
           (workloads.make_params(300, 600, 4500, 1e-3, 30, 8.0), 24)]
    alone = sum(plan_batch(p, n, cap // 2).est_seconds for p, n in big)
    assert fused_seconds(big, cap // 2) > alone


def test_admission_waits_rather_than_squeezing():
    """A batch planned in the little memory running calls leave (tiny waves)
    waits for them; with nothing running, or with room, it starts."""
    from geopvi_gb300 import workloads
    from geopvi_gb300.scheduler import plan_batch, worth_starting
    p = workloads.make_params(400, 800, 4363, 1e-3, 32, 8.0)
    best = plan_batch(p, 8, 150 << 30)
    squeezed = plan_batch(p, 8, 4 << 30)  # one resident solve, checkpointed
    assert best is not None and squeezed is not None
    assert squeezed.est_seconds > 3 * best.est_seconds
    assert not worth_starting(squeezed.est_seconds, best.est_seconds, True)
    assert worth_starting(squeezed.est_seconds, best.est_seconds, False)
    roomy = plan_batch(p, 8, 120 << 30)
    assert worth_starting(roomy.est_seconds, best.est_seconds, True)

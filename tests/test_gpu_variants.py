"""FD step kernel variants and the tuner that picks among them.

Every variant (rows per interior block x blocks per SM) computes the same
values bit for bit, so results never depend on the tuner's choice.
"""
import os

import numpy as np
import pytest
import torch

import cases
from geopvi_gb300 import _native

pytestmark = pytest.mark.gpu

GOLDEN = os.path.dirname(cases.__file__)


def run(p, vel, obs, **kw):
    from geopvi_gb300.engine import Fwi2dEngine
    eng = Fwi2dEngine(p, device="cuda:0", graph=False, **kw)
    v = torch.from_numpy(np.ascontiguousarray(np.atleast_2d(vel), dtype=np.float32)).cuda()
    o = torch.from_numpy(np.ascontiguousarray(obs, dtype=np.float32)).cuda()
    r = eng.run(v, o, want_syn=True)
    torch.cuda.synchronize()
    return eng, r.misfit.cpu().numpy().copy(), r.grad.cpu().numpy().copy(), r.syn.cpu().numpy().copy()


@pytest.mark.parametrize("name", ["fwi_o8", "fwi_o12", "fwi_ragged", "img_o6"])
def test_every_variant_is_bit_identical(engine_lib, cuda, name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    p = cases.params_from_npz(z)
    vel = np.stack([z["start"], z["truth"]]).astype(np.float32)
    ref = None
    for v in range(_native.NUM_STEP_VARIANTS):
        _, m, g, syn = run(p, vel, z["obs"], variant=v)
        if ref is None:
            ref = (m, g, syn)
            assert np.array_equal(syn[0], z["syn"])  # variant 0 against the reference's own data
        else:
            assert np.array_equal(m, ref[0]) and np.array_equal(g, ref[1]) and np.array_equal(syn, ref[2]), v


def test_tuner_settles_and_results_do_not_move(engine_lib, cuda):
    from geopvi_gb300.engine import Fwi2dEngine
    z = np.load(os.path.join(GOLDEN, "fwi_o8.npz"))
    p = cases.params_from_npz(z)
    eng = Fwi2dEngine(p, device="cuda:0", graph=False)
    v = torch.from_numpy(np.stack([z["start"], z["truth"]]).astype(np.float32)).cuda()
    o = torch.from_numpy(z["obs"].astype(np.float32)).cuda()
    outs = []
    for _ in range(_native.NUM_STEP_VARIANTS + 2):
        r = eng.run(v, o)
        torch.cuda.synchronize()
        outs.append(r.grad.cpu().numpy().copy())
    assert all(np.array_equal(outs[0], x) for x in outs[1:])
    chosen = eng.tuned_variant(2)
    assert 0 <= chosen < _native.NUM_STEP_VARIANTS
    with pytest.raises(_native.EngineError):
        run(p, z["start"], z["obs"], variant=_native.NUM_STEP_VARIANTS)


def test_tuner_tries_a_variant_per_wave(engine_lib, cuda):
    """Six waves of one solve: every variant is tried within the first call."""
    from geopvi_gb300.engine import Fwi2dEngine
    z = np.load(os.path.join(GOLDEN, "fwi_o8.npz"))
    p = cases.params_from_npz(z)
    eng = Fwi2dEngine(p, device="cuda:0", graph=True, max_resident=1)
    v = torch.from_numpy(np.stack([z["start"], z["truth"]]).astype(np.float32)).cuda()
    o = torch.from_numpy(z["obs"].astype(np.float32)).cuda()
    g0 = eng.run(v, o).grad.cpu().numpy().copy()
    torch.cuda.synchronize()
    assert 0 <= eng.tuned_variant(2) < _native.NUM_STEP_VARIANTS
    g1 = eng.run(v, o).grad.cpu().numpy().copy()  # the tuned variant, now through a CUDA graph
    assert np.array_equal(g0, g1)
    ref = Fwi2dEngine(p, device="cuda:0", graph=False, variant=0).run(v, o).grad.cpu().numpy()
    assert np.array_equal(g0, ref)

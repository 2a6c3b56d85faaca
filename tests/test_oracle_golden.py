"""The oracle restatement against the reference's own outputs (CPU only).

The fixtures in tests/golden were produced by the reference solver compiled
unmodified from its C sources (tests/golden/make_golden.py).  The FP32
restatement must reproduce them bit for bit; the FP64 restatement must agree
to FP32 round-off.
"""
import hashlib
import os

import numpy as np
import pytest

import cases

GOLDEN = os.path.dirname(cases.__file__)


def load(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def oparams(O, p):
    return O.Params(**cases.params_to_dict(p))


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", sorted(cases.SMALL))
def test_restatement_bitwise(oracle, name):
    z = load(name)
    p = cases.params_from_npz(z)
    op = oparams(oracle, p)
    obs = oracle.forward_f32(op, z["truth"])
    assert np.array_equal(obs, z["obs"]), "forward data differ from the reference"
    syn, grad = oracle.fwi_f32(op, z["start"], z["obs"], int(z["run_fwi"]))
    assert np.array_equal(syn, z["syn"]), "synthetic data differ from the reference"
    assert np.array_equal(grad, z["grad"]), "gradient differs from the reference"


@pytest.mark.parametrize("name", sorted(cases.SMALL))
def test_fp64_restatement_close(oracle, name):
    z = load(name)
    p = cases.params_from_npz(z)
    op = oparams(oracle, p)
    syn, grad = oracle.fwi_f64(op, z["start"].astype(np.float64), z["obs"].astype(np.float64),
                               int(z["run_fwi"]))
    assert rel(syn, z["syn"]) < 1e-4
    assert rel(grad, z["grad"]) < 1e-3


def test_ricker_matches_reference_definition(oracle):
    # getrik (fdtd2D_modelling.c:1084-1093) at the benchmark's first config
    rik = oracle.ricker_f32(2000, 1e-3, 10.0)
    assert rik.dtype == np.float32 and rik.shape == (2000,)
    assert abs(float(rik[100]) - 1.0) < 1e-6          # peak at t = 1/f0
    assert np.argmax(rik) == 100


def test_paramfile_roundtrip(oracle, tmp_path):
    p = cases.SMALL["fwi_ragged"]["params"]
    path = str(tmp_path / "p.txt")
    op = oparams(oracle, p)
    oracle.write_paramfile(path, op)
    back = oracle.read_params(path)
    for f in oracle.INT_FIELDS:
        assert getattr(back, f) == getattr(op, f), f
    for f in oracle.FLOAT_FIELDS:  # the file is parsed with %f into a float
        assert np.float32(getattr(back, f)) == np.float32(getattr(op, f)), f


@pytest.mark.slow
@pytest.mark.parametrize("name", sorted(cases.FULL))
def test_full_size_forward_hash(oracle, name):
    """Full-size forward data of the restatement hash-equal to the reference's."""
    path = os.path.join(GOLDEN, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip("full-size fixture not generated")
    z = np.load(path)
    p = cases.params_from_npz(z)
    obs = oracle.forward_f32(oparams(oracle, p), z["truth"])
    assert hashlib.sha256(obs.tobytes()).hexdigest() == str(z["obs_sha256"])

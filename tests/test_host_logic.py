"""Host-side logic of the drop-in API against golden vectors produced by the
reference's own Python (tests/golden/make_golden.py): the FP64 operator build
and particle generation.  No kernel is called (tensors live on the CPU)."""
from copy import deepcopy

import numpy as np
import pytest

from conftest import rel_l2

import sys, os  # noqa: E401
sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))


def _configs():
    from make_golden import solver_configs
    return solver_configs()


@pytest.mark.parametrize("name", ["lpa_m2", "lpa_m3_chunked", "plain_m1_vacuum", "fel_env_k1"])
def test_operator_build_matches_reference(golden, name):
    from chimera_gb300.solvers import Solver
    from chimera_gb300.messages import msg
    msg.quiet = True
    s = Solver(deepcopy(_configs()[name]), device="cpu")
    pre = f"op/{name}/Args/"
    keys = [k[len(pre):] for k in golden.files if k.startswith(pre)]
    assert keys
    for k in keys:
        ref = golden[pre + k]
        got = np.asarray(s.Args[k])
        assert got.shape == ref.shape, k
        if ref.dtype.kind in "fc":
            assert rel_l2(got, ref) <= 1e-15 or np.array_equal(got, ref), k
        else:
            assert np.array_equal(got, ref), k
    for k in ("PSATD_E", "PSATD_G"):
        ref = golden[f"op/{name}/Data/{k}"]
        got = s.Data[k].numpy()
        assert got.shape == ref.shape and rel_l2(got, ref) < 1e-15, k
    if name == "lpa_m2":
        assert np.array_equal(s.get_damp_profile(12), golden["op/lpa_m2/damp_profile"])


def test_gen_parts_matches_reference(golden):
    from chimera_gb300.species import Specie
    np.random.seed(7)
    sp = Specie({"Grid": (-2.0, 1.0, 2.0, 0.1, 0.25), "TimeStep": 0.1, "Density": 0.01,
                 "FixedCell": (2, 2, 3), "MomentaSpreads": (0.1, 0.05, 0.05)}, device="cpu")
    c, p, w = sp.gen_parts(Domain=(-1.5, 0.8, 0.0, 1.5),
                           ProfileFunc=lambda x, r: np.exp(-r ** 2) * (1 + 0.1 * x))
    assert c.shape == golden["gen/fixed/coords"].shape
    assert rel_l2(c, golden["gen/fixed/coords"]) < 1e-15
    assert np.array_equal(p, golden["gen/fixed/momenta"])
    assert rel_l2(w, golden["gen/fixed/weights"]) < 1e-15
    c, p, w = sp.gen_parts(Xsteps=3)
    assert rel_l2(c, golden["gen/xsteps/coords"]) < 1e-15
    assert np.array_equal(p, golden["gen/xsteps/momenta"])


def test_particle_store_append_and_permute_host():
    import torch
    from chimera_gb300.species import ParticleStore
    st = ParticleStore({"a": 3, "w": 1}, torch.device("cpu"), capacity=4)
    st.append({"a": np.arange(15.).reshape(3, 5), "w": np.arange(5.)})
    assert st.n == 5 and st.cap >= 5
    v = st.views()
    assert v["a"].shape == (3, 5) and v["w"].shape == (5,)
    assert v["a"].stride() == (st.cap, 1)


def test_moving_frame_defaults():
    from chimera_gb300.chimera_main import ChimeraRun
    run = ChimeraRun.__new__(ChimeraRun)
    run.MovingFrames = ({}, {"Features": ("Staged",), "Velocity": 0.5, "TimeStep": 0.1,
                             "Steps": 2})
    run.init_Moving_Frames()
    assert run.MovingFrames[0]["shiftX"] == 1.0
    assert abs(run.MovingFrames[1]["shiftX"] - 0.05) < 1e-15

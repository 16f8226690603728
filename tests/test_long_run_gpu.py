"""Long-horizon accuracy of the split-precision form: the 512 x 64 x 2-mode
laser-wakefield workload (chimera_gb300/workloads.py, with the window's
plasma injection, AddPlasma + AbsorbLayer + IonsOnTop) advanced 500 steps in
the split form and in the plain FP64 form from the same particles, laser and
injected plasma.  The observables of the reference's demos must agree within
1 % along the run: the wake amplitude max |Re E_x| on the axis (mode 0,
first row) and the laser amplitude max Re E_z of mode 0 on the ghost row, as
the LPA demo records it (doc/fel-lpa-demo.ipynb, laser_amplitude)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
STEPS = 500
TOL_OBS = 0.01


def _obs(EB):
    wake = float(EB[:, 1, 0, 0].real.abs().max())
    a0 = float(EB[:, 0, 0, 2].real.max())
    return wake, a0


def test_lwfa_500_steps_split_tracks_fp64(cuda):
    import torch
    from chimera_gb300 import ChimeraRun, _lib, workloads
    from chimera_gb300.split import SplitRun
    fp = ChimeraRun(workloads.components("cfg1", "inject", seed=1001))
    sp = SplitRun(workloads.components("cfg1", "inject", seed=1001))
    worst = {"wake": 0.0, "a0": 0.0}
    rows = []
    for i in range(1, STEPS + 1):
        np.random.seed(7000 + i)  # the same injected plasma in both forms
        fp.make_step(i)
        np.random.seed(7000 + i)
        sp.make_step(i)
        if i % 50 == 0:
            w64, a64 = _obs(fp.Solvers[0].Data["EB"])
            w32, a32 = _obs(sp.EB)
            dw, da = abs(w32 - w64) / abs(w64), abs(a32 - a64) / abs(a64)
            worst["wake"] = max(worst["wake"], dw)
            worst["a0"] = max(worst["a0"], da)
            rows.append((i, w64, w32, a64, a32))
    torch.cuda.synchronize()
    for r in rows:
        print("step %d: wake %.6g / %.6g  a0 %.6g / %.6g (fp64 / split)" % r)
    print(f"worst relative deviation over {STEPS} steps: wake {worst['wake']:.2e}, "
          f"a0 {worst['a0']:.2e}")
    assert rows[-1][1] > 0 and rows[-1][3] > 0
    assert worst["wake"] < TOL_OBS and worst["a0"] < TOL_OBS, worst
    assert sp.num_moving > 0
    sp.check_status()
    assert _lib.load().chm_sp_umma_status() == 0

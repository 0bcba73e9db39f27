"""Every code path through the bounds-checked build (field indices checked
and clamped on the device, violations recorded in each instance's status
word), on small and ragged grids: no index may leave its field.  This
stands in for an external memory checker, which these tests do not run."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import sys, tempfile, os
from dataclasses import replace
import numpy as np
from channel_rl_gb300 import cases as C
from channel_rl_gb300.host import Channel

def report(tag, ch, n):
    for q in range(n):
        print(f"FLAGS {tag} {q} {ch.status_flags(q)}")

tmp = tempfile.mkdtemp()
# batched dynamic Smagorinsky + equilibrium wall model, every entry point
batch = [C.smaller(C.c2_wm64(), 32, 16, 16), C.smaller(C.c3_roofline(les=C.LES_DSM), 24, 9, 36),
         C.wallmodelled("b", 6, 8, 4, 3000.0, x_mass_cte=1)]
ch = Channel(batch)
for q, c in enumerate(batch):
    ch.upload(*C.initial_fields(c), inst=q)
ch.step(2)
ch.compute_eddy_viscosity(); ch.compute_wall_model(); ch.compute_projection_step(); ch.compute_pressure()
for q in range(len(batch)):
    ch.compute_statistics(q); ch.check_divergence(q); ch.compute_rhs(q)
    ch.compute_dPx_for_constant_mass_flow(q); ch.pseudo_pressure(q)
ch.save_snapshot(os.path.join(tmp, "s"), inst=1)
ch.synchronize()
report("dsm_batch", ch, len(batch))
ch.close()
# the other SGS models and ghost rules, no wall model and stress wall model
for les, dn, wm in ((C.LES_SMAG, 0, C.WM_EQLOG), (C.LES_AMD, 2, C.WM_EQLOG), (C.LES_VREMAN, 1, C.WM_NONE),
                    (C.LES_NONE, 1, C.WM_STRESS), (C.LES_AMD, 0, C.WM_NONE)):
    c = replace(C.smaller(C.c3_roofline(les=C.LES_DSM), 18, 10, 12), LES_model=les, Dirichlet_nu_t=dn,
                wall_model=wm)
    ch = Channel(c)
    ch.upload(*C.initial_fields(c))
    ch.step(3)
    ch.compute_pressure(); ch.compute_statistics()
    report(f"les{les}_d{dn}_wm{wm}", ch, 1)
    ch.close()
# learned wall model with exploration and the policy-gradient trace
b5 = [C.wallmodelled("m0", 32, 16, 16, 2000.0, wall_model=C.WM_MLP),
      C.wallmodelled("m1", 12, 8, 36, 10000.0, wall_model=C.WM_MLP)]
ch = Channel(b5)
for q, c in enumerate(b5):
    ch.upload(*C.initial_fields(c), inst=q)
ch.mlp_configure(sigma=0.1, seed=3, train=True)
ch.step(2)
ch.mlp_trace(0); ch.mlp_trace(1)
report("mlp", ch, len(b5))
ch.close()
# wall agents of the RL protocol (reference mesh convention, walls at 0 and 2)
c0 = C.wallmodelled("ag", 32, 16, 16, 2000.0, wall_model=C.WM_STRESS)
x, y, z = C.faces(c0)
c = replace(c0, xf=tuple(x), yf=tuple(y + 1.0), zf=tuple(z))
ch = Channel(c)
ch.upload(*C.initial_fields(c0))
ch.step(1)
ch.agent_observe(8, np.full((2, 8), 4), np.full((2, 8), 0.5))
ch.agent_act(8, np.full((2, 8), 1.05))
ch.step(1)
report("agents", ch, 1)
ch.close()
print("DONE")
'''


def test_every_path_stays_in_bounds():
    from channel_rl_gb300 import build
    lib = build.build(variant="bounds")
    env = dict(os.environ, CHL_LIBRARY=lib)
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    flags = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("FLAGS")]
    assert "DONE" in r.stdout and len(flags) >= 11
    bad = [f for f in flags if int(f[3]) != 0]
    assert not bad, bad

"""The reference's RL environment protocol over one channel instance.

The reference runs one smarties environment per solver process: every step
of the app_main loop (app_main.f90:108-127) first calls
send_recv_state_action (smarties_stat.f90:24-260), which

* at step 1 computes the eddy viscosity and sets the wall stress alpha_x to
  dPdx_ref (1 + (aa - 1/2)) with one random aa;
* at step 1000 sends every agent's initial state and receives its action;
* every 200 steps after that (before nsteps) sends state and reward and
  receives a new action; at nsteps sends the last state;
* from step 1000 on rebuilds alpha_x from the actions: the action multiplies
  the current wall stress at the agent, and alpha_x is interpolated linearly
  in x between agents (chl_agent_act).

The reward sent is r - r_old, plus r when r > 0, with
r = 100 - 5000 |u_tau - sqrt(dPdx_ref)| / sqrt(dPdx_ref) per agent.  The
state has six entries of which the reference lets smarties observe the
first two (app_main.f90:92-98).  `WallAgentEnv` reproduces that schedule;
the policy is any callable (smarties is not part of this project), bounded
to the reference's action range [0.9, 1.1] (app_main.f90:84-88).
"""
from __future__ import annotations

import numpy as np

from .host import Channel

ACTION_LOW, ACTION_HIGH = 0.9, 1.1
FIRST_DECISION, DECISION_EVERY = 1000, 200


class WallAgentEnv:
    def __init__(self, channel: Channel, case, nagents=128, seed=0, inst=0):
        if case.Nx % nagents:
            raise ValueError("nagents must divide Nx")
        self.ch, self.case, self.nagents, self.inst = channel, case, nagents, inst
        self.rng = np.random.default_rng(seed)
        self.dPdx_ref = case.dPdx
        self.rewards_old = None
        self.decisions = 0

    def draws(self):
        """The sampling rows and weights: per agent and wall, y_ind = 3 or 4
        with probability 1/2 each and a uniform weight, the two
        RANDOM_NUMBER draws of smarties_stat.f90:63-69 and :108-114."""
        u = self.rng.random((2, self.nagents, 2))
        return np.where(u[..., 0] < 0.5, 3, 4).astype(np.int32), u[..., 1]

    def observe(self):
        y_ind, y_rand = self.draws()
        return self.ch.agent_observe(self.nagents, y_ind, y_rand, inst=self.inst)

    def shaped_reward(self, r):
        """reward = r - r_old, plus r where r > 0 (smarties_stat.f90:205-209)."""
        out = r - self.rewards_old
        return np.where(r > 0.0, out + r, out)

    def run(self, nsteps, policy, on_send=None):
        """The app_main step loop for nsteps steps.  policy(observed_states,
        reward_or_None) -> actions [2][nagents]; on_send(istep, states,
        reward, last) sees every message the reference would send."""
        for istep in range(1, nsteps + 1):
            if istep == 1:
                self.ch.compute_eddy_viscosity()
                aa = self.rng.random()
                a = np.full((self.case.nx, 2, self.case.nz + 1), self.dPdx_ref * (1.0 + (aa - 0.5)), order="F")
                self.ch.set_wall_stress(a, inst=self.inst)
            send = istep == FIRST_DECISION or istep == nsteps or \
                (FIRST_DECISION < istep < nsteps and istep % DECISION_EVERY == 0)
            if send and istep >= FIRST_DECISION:
                states, r = self.observe()
                reward = None if istep == FIRST_DECISION else self.shaped_reward(r)
                last = istep == nsteps
                if on_send is not None:
                    on_send(istep, states, reward, last)
                if not last:
                    act = np.clip(np.asarray(policy(states[..., :2], reward), dtype=np.float64),
                                  ACTION_LOW, ACTION_HIGH)
                    self.ch.agent_act(self.nagents, act, inst=self.inst)
                    self.decisions += 1
                self.rewards_old = r
            self.ch.step(1)
        self.ch.synchronize()

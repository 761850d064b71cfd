"""Time stepping of the shell: activation ramps and the implicit time loop.

The activation law is GammaOfTimeDelayed (active_strain.c:1156-1179): at
step ti the element's fibre contraction is

    gamma_e(ti) = G(ti * dt - delay_e) * gamma_scale_e          (ElemActDefGrad,
                                                                  active_strain.c:1207-1212)

with G one of
    0  constant gamma
    1  gamma sin^2(pi t / T)               (a full cycle, T = gamma_T or tisteps * dt)
    2  gamma sin^2(pi t / (2 T))           (systole only)
    3  gamma phi_up(t) phi_down(t)         (double-logistic pulse: tau_up, tau_down, APD)
and G = 0 for t <= 0 in ramps 1 and 2.

The time loop is main.c:420-573 for one body with the implicit solver:
per step, the activation of that step, a Newton solve from the previous
positions with the dynamic term (FDynamic) in the residual, then xAccVel
and xnm1 <- xn, xn <- x.  A step whose Newton solve fails keeps the
previous positions (main.c:501-529) and still advances the state.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .gpu import BiofemError, GpuShell


@dataclass
class Activation:
    """The -gamma / -gamma_ramp_type / -gamma_T / -gamma_tau_up /
    -gamma_tau_down / -gamma_apd options."""
    gamma: float
    ramp_type: int = 0
    T: float = 0.0
    tau_up: float = 0.0
    tau_down: float = 0.0
    apd: float = 0.0

    def __post_init__(self):
        if self.ramp_type not in (0, 1, 2, 3):
            raise ValueError(f"unknown gamma ramp type {self.ramp_type}")

    def at(self, ti: int, dt: float, tisteps: int, delay=0.0):
        """G(ti * dt - delay); ``delay`` may be a per-element array."""
        delay = np.asarray(delay, dtype=np.float64)
        if self.ramp_type == 0:
            return np.full(delay.shape, self.gamma) if delay.ndim else float(self.gamma)
        t = float(ti) * dt - delay
        if self.ramp_type == 3:
            tau_up = self.tau_up if self.tau_up > 0.0 else 0.02
            tau_down = self.tau_down if self.tau_down > 0.0 else 0.08
            apd = self.apd if self.apd > 0.0 else 0.30
            t_up = 4.0 * tau_up
            t_down = t_up + apd
            phi_up = 1.0 / (1.0 + np.exp(-(t - t_up) / tau_up))
            phi_down = 1.0 / (1.0 + np.exp((t - t_down) / tau_down))
            g = self.gamma * phi_up * phi_down
        else:
            T = self.T if self.T > 0.0 else float(tisteps) * dt
            arg = (np.pi * t / T) if self.ramp_type == 1 else (np.pi * 0.5 * t / T)
            s = np.sin(arg)
            g = np.where(t <= 0.0, 0.0, self.gamma * s * s)
        return g if delay.ndim else float(g)

    def element_gamma(self, ti: int, dt: float, tisteps: int, gamma_scale, delay=None) -> np.ndarray:
        gs = np.asarray(gamma_scale, dtype=np.float64)
        d = np.zeros_like(gs) if delay is None else np.asarray(delay, dtype=np.float64)
        return self.at(ti, dt, tisteps, d) * gs


@dataclass
class Dynamics:
    """The -dt, -rho, -newmark_gamma, -dampfactor, -timeinteg, -damping options.
    timeinteg 0 is Newmark with Beta = (gamma + 1/2)^2 / 4, 1 central differences."""
    dt: float
    rho: float
    newmark_gamma: float = 0.5
    dampfactor: float = 0.0
    timeinteg: int = 0
    damping: int = 0

    def apply(self, shell) -> None:
        shell.set_dynamics(self.dt, self.rho, self.newmark_gamma, self.dampfactor, self.timeinteg, self.damping)


@dataclass
class StepRecord:
    ti: int
    gamma_mean: float
    converged: bool
    stats: dict = field(default_factory=dict)


def time_loop(shell: GpuShell, mesh, x0: np.ndarray, dyn: Dynamics, act: Activation, tisteps: int,
              tistart: int = 0, delay=None, on_step=None, pre_update=None, reset_state: bool = True, **newton):
    """Run ``tisteps`` implicit steps (ti = tistart .. tistart + tisteps - 1) from
    x0 on a prepared GpuShell.

    ``pre_update(ti, x)`` is called with the step's solution before xAccVel,
    ``on_step(ti, x, record)`` after it (for output).  ``reset_state`` = False
    keeps the dynamic state already on the shell (a restart).  The ramps'
    default period is ``tisteps * dt`` as in the reference, where tisteps is
    the run's step count.  Returns (x, [StepRecord]).
    """
    if reset_state:
        dyn.apply(shell)
    x = np.array(x0, dtype=np.float64, copy=True)
    records = []
    for ti in range(tistart, tistart + tisteps):
        g = act.element_gamma(ti, dyn.dt, tisteps, mesh.gamma_scale, delay)
        shell.set_element_gamma(g)
        try:
            x_new, st = shell.newton(x, **newton)
            ok = True
        except BiofemError as e:
            x_new, st, ok = x, dict(getattr(e, "stats", {}) or {}, error=str(e)), False
        x = x_new
        if pre_update is not None:
            pre_update(ti, x)
        shell.dynamic_update(x)
        rec = StepRecord(ti, float(np.mean(g)), ok, st)
        records.append(rec)
        if on_step is not None:
            on_step(ti, x, rec)
    return x, records

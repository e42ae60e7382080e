"""The P-E loop schedule of the reference driver.

``evolve_schedule`` restates the control flow of ``Evolve``
(HZO_Code_github/src/evolve.cu:213-409) without any field arithmetic: the
applied field is a staircase that holds each value for ``num_steps`` TDGL
steps, reverses above +Emax / below -Emax, and the loop ends at the second
reversal above +Emax (``peloop < 2``, :217).  Sweep rows are written after
the first reversal.  The field only depends on these counters, so the whole
schedule is known before the first step; the GPU engine consumes it as two
device arrays (applied field per step, output row per step).

The same additions as the reference are made in the same order
(``Ez_ext += incEz``, :407), so every field value is bit-identical to the
reference's.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Schedule:
    Ez: np.ndarray        # [n_steps] applied non-dimensional field per step
    rows: np.ndarray      # [n_steps] output row index or -1
    row_E: np.ndarray     # [n_rows] field printed in each row (non-dimensional)
    row_count: np.ndarray  # [n_rows] the reference's `count` printed in each row

    @property
    def n_steps(self) -> int:
        return int(self.Ez.size)

    @property
    def n_rows(self) -> int:
        return int(self.row_E.size)


def evolve_schedule(maxEz: float, delEz: float, num_steps: int, *, n_periods: int = 1,
                    crystal_single: bool = False, E0_ref: float = 1.0, count0: int = 0,
                    max_steps: int = 50_000_000) -> Schedule:
    """Restates evolve.cu:123-409.  ``n_periods`` = 1 is the reference's
    ``peloop < 2``; larger values record more periods (the loop ends when
    ``peloop`` reaches ``n_periods + 1``)."""
    if delEz <= 0 or num_steps < 1:
        raise ValueError("delEz must be > 0 and num_steps >= 1")
    Ez_ext = 0.0                       # reset_evolve_state, main.cu:66-70
    incEz = delEz                      # evolve.cu:123
    peloop = 0
    count = count0
    steps_since_change = 0
    base = num_steps                   # time_to_change = num_steps, main.cu:354
    Ewin_nd = 0.2e8 / E0_ref           # evolve.cu:243
    Ez_list, rows = [], []
    row_E, row_count = [], []
    while peloop < n_periods + 1:
        Ez_list.append(Ez_ext)
        rows.append(-1)
        steps_since_change += 1
        count += 1
        relax = base
        if crystal_single and abs(Ez_ext) < Ewin_nd:   # evolve.cu:245-249
            relax = base * 10
        if steps_since_change >= relax:
            if Ez_ext > maxEz:                          # evolve.cu:362-369
                incEz = -delEz
                peloop += 1
            if Ez_ext < -maxEz:
                incEz = delEz
            if peloop > 0:                              # evolve.cu:390-403
                rows[-1] = len(row_E)
                row_E.append(Ez_ext)
                row_count.append(count)
            Ez_ext += incEz                             # evolve.cu:407
            steps_since_change = 0
        if len(Ez_list) > max_steps:
            raise ValueError("schedule does not terminate within max_steps")
    return Schedule(np.asarray(Ez_list, np.float64), np.asarray(rows, np.int32),
                    np.asarray(row_E, np.float64), np.asarray(row_count, np.int64))


def triangle_schedule(E_amp: float, steps_per_period: int, n_periods: int = 1) -> Schedule:
    """A triangle wave of amplitude E_amp and steps_per_period steps, run as the
    reference runs it: num_steps = 1, delEz = 4 E_amp / steps_per_period, an
    unrecorded quarter-period ramp, then n_periods recorded periods."""
    return evolve_schedule(E_amp, 4.0 * E_amp / steps_per_period, 1, n_periods=n_periods)


def constant_schedule(E: float, n_steps: int, row_every: int = 0) -> Schedule:
    """A fixed field for n_steps steps; a row every `row_every` steps (0: none)."""
    Ez = np.full(n_steps, float(E))
    rows = np.full(n_steps, -1, np.int32)
    row_E, row_count = [], []
    if row_every > 0:
        for s in range(row_every - 1, n_steps, row_every):
            rows[s] = len(row_E)
            row_E.append(float(E))
            row_count.append(s + 1)
    return Schedule(Ez, rows, np.asarray(row_E, np.float64), np.asarray(row_count, np.int64))


def sweep_lines(rows: np.ndarray, sched: Schedule, E0_ref: float, P0_ref: float) -> list[str]:
    """The reference's sweep-file lines (evolve.cu:391-400): E in MV/cm, P in
    uC/cm^2, then the count; fields tab-separated in C's %le format."""
    Ez_scale = E0_ref / 1.0e+08
    P0_scale = P0_ref * 100.0
    out = []
    for r in range(sched.n_rows):
        v = rows[r]
        vals = [sched.row_E[r] * Ez_scale, v[0] * P0_scale, v[1] * P0_scale, v[2] * P0_scale,
                v[3] * P0_scale, v[4] * P0_scale, v[5], v[6] * P0_scale, v[7], v[8] * P0_scale, v[9]]
        out.append("\t".join("%e" % x for x in vals) + "\t%d" % int(sched.row_count[r]))
    return out

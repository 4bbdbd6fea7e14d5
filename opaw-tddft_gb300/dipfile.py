"""Dipole time series in the reference's files (plot_dip, tddft_plot.f90:62-105).

Per step `it` (1-based) of a run the reference appends

  d_dip.dat   format (' ',4e18.8):   (it-1) dt, d_dip(1:3)
  dip.dat     list-directed:         (it-1) dt, dip(1:3), dip_pert(1:3)

and a run restarted from step it_restart (tddft_save/info) continues them:

* d_dip_cont.dat exists (an earlier restart):  append to it and dip_cont.dat;
* else d_dip.dat exists:  create d_dip_cont.dat / dip_cont.dat holding the
  first it_restart lines of d_dip.dat / dip.dat, then append.  The copied
  dip lines keep only their first four values, t and dip(1:3): the
  reference reads them back with `read(19,*) tmp, tmp3d` and writes what it
  read (tddft_plot.f90:77-82);
* else:  start d_dip.dat / dip.dat afresh.

`DipoleLog` follows those rules; `read_series` reads any of the four files.
Host-side code: no GPU.
"""
from __future__ import annotations

import math
import os
import re

import numpy as np


def fortran_e(x: float, w: int = 18, d: int = 8) -> str:
    """One value in Fortran's Ew.d edit descriptor: 0.d1..dd E+xx, right
    justified in w characters; exponents beyond 99 drop the E (+xxx)."""
    x = float(x)
    if not math.isfinite(x):
        return ("NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")).rjust(w)
    if x == 0.0:
        digits, e = "0" * d, 0
    else:
        s = f"{abs(x):.{d - 1}e}"  # d significant digits, correctly rounded
        mant, ex = s.split("e")
        digits = mant.replace(".", "")
        e = int(ex) + 1
    sign = "-" if x < 0 else ""
    exp = f"E{'+' if e >= 0 else '-'}{abs(e):02d}" if abs(e) <= 99 else f"{'+' if e >= 0 else '-'}{abs(e):03d}"
    field = f"{sign}0.{digits}{exp}"
    return field.rjust(w) if len(field) <= w else "*" * w


def format_d_dip_line(t, d_dip) -> str:
    """One d_dip.dat line, format (' ',4e18.8)."""
    return " " + "".join(fortran_e(v) for v in (t, *d_dip)) + "\n"


def format_list_line(values) -> str:
    """A list-directed output line: blank-separated values with 17
    significant digits (any such line reads back with list-directed input)."""
    return "".join(f" {float(v):24.16E}" for v in values) + "\n"


_FEXP = re.compile(r"(?<=[0-9.])([+-]\d{3})$")


def _parse_value(tok: str) -> float:
    tok = tok.replace("D", "E").replace("d", "e")
    return float(_FEXP.sub(r"E\1", tok))


def read_series(path):
    """All values of a dipole file as a [lines, values] array (lines of
    unequal length keep their leading values, padded with NaN)."""
    rows = []
    with open(path) as f:
        for line in f:
            toks = line.split()
            if toks:
                rows.append([_parse_value(t) for t in toks])
    if not rows:
        return np.zeros((0, 0))
    width = max(len(r) for r in rows)
    out = np.full((len(rows), width), np.nan)
    for i, r in enumerate(rows):
        out[i, :len(r)] = r
    return out


class DipoleLog:
    """The dipole files of one run.  dt: the time step; it_restart: the step a
    restarted run starts after (None for a fresh run)."""

    def __init__(self, dt, directory=".", it_restart=None):
        self.dt = float(dt)
        self.dir = directory
        self.it_restart = it_restart
        self.f15 = self.f16 = None

    def _path(self, name):
        return os.path.join(self.dir, name)

    def _open(self, it):
        if self.it_restart is not None and self.it_restart > 0:
            if it != self.it_restart + 1:
                raise ValueError(f"a run restarted after step {self.it_restart} starts at step "
                                 f"{self.it_restart + 1}, not {it}")
            if os.path.exists(self._path("d_dip_cont.dat")):
                self.f15 = open(self._path("d_dip_cont.dat"), "a")
                self.f16 = open(self._path("dip_cont.dat"), "a")
            elif os.path.exists(self._path("d_dip.dat")):
                dd = read_series(self._path("d_dip.dat"))
                dp = read_series(self._path("dip.dat"))
                n = self.it_restart
                if dd.shape[0] < n or dp.shape[0] < n or dd.shape[1] < 4 or dp.shape[1] < 4:
                    raise ValueError(f"d_dip.dat / dip.dat hold fewer than the {n} steps to continue from")
                self.f15 = open(self._path("d_dip_cont.dat"), "w")
                self.f16 = open(self._path("dip_cont.dat"), "w")
                for i in range(n):
                    self.f15.write(format_d_dip_line(dd[i, 0], dd[i, 1:4]))
                    self.f16.write(format_list_line(dp[i, :4]))
            else:
                self._fresh()
        else:
            if it != 1:
                raise ValueError(f"a fresh run starts at step 1, not {it}")
            self._fresh()

    def _fresh(self):
        os.makedirs(self.dir, exist_ok=True)
        self.f15 = open(self._path("d_dip.dat"), "w")
        self.f16 = open(self._path("dip.dat"), "w")

    def write(self, it, d_dip, dip, dip_pert):
        """Step it (1-based) of the run."""
        if self.f15 is None:
            self._open(it)
        t = (it - 1) * self.dt
        self.f15.write(format_d_dip_line(t, d_dip))
        self.f16.write(format_list_line((t, *dip, *dip_pert)))
        self.f15.flush()
        self.f16.flush()

    def write_steps(self, it0, dip, dip_pert, d_dip):
        """Steps it0+1 .. it0+n from the [n, 3] arrays of
        Context.tddft_steps_dip."""
        for k in range(len(d_dip)):
            self.write(it0 + 1 + k, d_dip[k], dip[k], dip_pert[k])

    def close(self):
        for f in (self.f15, self.f16):
            if f is not None:
                f.close()
        self.f15 = self.f16 = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

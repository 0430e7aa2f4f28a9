"""Driver: configuration, time loop and history (drop-in for pylbm_isca/model.py).

``LBM.run`` has two loops with the reference's step semantics
(model.py:213-290):

* the fused loop (default): the whole ensemble advances in the lbm_gb300
  fused stepper with the state in packed spectral space; steady-state steps
  replay as CUDA graphs; the blow-up check reads a device flag once per
  model day instead of synchronising every step, and reports the day in
  which a non-finite value appeared; with a history writer the stepper
  accumulates the trapezoid of the spectral state and grid ps' each step
  and the daily fields are formed once per day from the mean;
* the general loop (a history writer with a non-zero initial state, or
  ``Config.fused=False``): one call of
  ``Dynamics.tendencies``, ``State.to_spectral``, ``Integrator.step``,
  ``State.load_spectral`` and the Robert-Asselin filter per step, each
  backed by the library's reference-layout kernels, exactly as the
  reference sequences them.

A non-zero initial state may not be band-limited, so the first call of a
fused run from one is made by the general step; every later state is
produced by the model and is band-limited except ps, whose grid values the
stepper keeps.
"""

from __future__ import annotations

import time as _time
from dataclasses import dataclass, field

import types

import numpy as np
import torch

from .backend import asnumpy, device_name
from .constants import GRAV
from .dynamics import BasicStateTerms, Dynamics
from .forcing import SpectralInterpolation
from .integrator import Damping, Integrator, SemiImplicit, VerticalDiffusion
from .state import State

# &nmdamp profile (model.py:30-31), days, k = 0 at the bottom
DDRAG_DEFAULT = [0.5, 0.5, 0.5, 5, 15, 20, 20, 20, 20, 20,
                 20, 20, 20, 20, 20, 20, 20, 20, 0.5, 0.5]


def _emit(writer, day, fields):
    """One history record: device tensors to a writer that takes them (the
    GrADS writer packs its records on the device), host arrays otherwise."""
    if getattr(writer, "accepts_device", False):
        writer.add(day, dict(fields))
    else:
        writer.add(day, {k: asnumpy(v) for k, v in fields.items()})


@dataclass
class Config:
    """The reference's namelist knobs (model.py:34-86) plus GB300 switches."""
    delt: float = 1200.0
    inistp: int = 2
    ndays: float = 66.0
    hdif_order: int = 4
    hdif_tefold: float = 2.0
    hdif_tunit: str = "HOUR"
    sponge: bool = True
    ray0: float = 30.0
    ddragv: list = field(default_factory=lambda: list(DDRAG_DEFAULT))
    ddragd: list = field(default_factory=lambda: list(DDRAG_DEFAULT))
    ddragt: list = field(default_factory=lambda: list(DDRAG_DEFAULT))
    ddragq: list = None
    damp_tunit: str = "DAY"
    vdifv: float = 1.0e3
    vdifd: float = 1.0e3
    vdift: float = 1.0e3
    vdifq: float = None
    robert: float = 0.04
    out_interval_days: float = 1.0
    time_average: bool = True
    strictly_linear: bool = False
    nmem: int = 1
    device: str = "auto"
    # --- GB300 path ----------------------------------------------------------
    precision: str = "fp64"       # "fp64" | "fp32" | "bf16x3" | "bf16split": working
                                  # precision of the step; the bf16 modes keep the FP32
                                  # state and run contractions on the tensor cores
                                  # (bf16 split, 6 or 3 products): bf16x3 the
                                  # longitude analysis, bf16split all three
    tc_off: int = -1              # bf16 modes: contractions kept on the FMA pipes (bit 0
                                  # Legendre analysis, 1 synthesis, 2 longitude
                                  # analysis); -1: the precision's default
    fused: bool = True            # fused ensemble stepper (False: general loop)
    use_graph: bool = True        # replay steady-state steps as CUDA graphs
    phase_timing: bool = False    # fused run: seconds per phase in LBM.phases
                                  # (synchronises the device at phase boundaries)

    @property
    def steps_per_day(self):
        return int(round(86400.0 / self.delt))

    @classmethod
    def from_namelist(cls, path):
        raise NotImplementedError(
            "namelist files are outside the GB300 hot path; build a Config directly")


class LBM:
    """Linear baroclinic model on one GB300 (model.py:89-290)."""

    def __init__(self, basic_state, spectral, vertical, config=None, basic_spectral=None):
        self.cfg = config or Config()
        self.sp = spectral
        self.vg = vertical
        self.bs = basic_state
        self.xp = torch
        self.bst = BasicStateTerms(basic_spectral or self.sp, self.vg, basic_state)
        self.dyn = Dynamics(self.sp, self.vg, self.bst, strictly_linear=self.cfg.strictly_linear)
        c = self.cfg
        self.damping = Damping(self.sp, self.vg, order=c.hdif_order, tefold=c.hdif_tefold,
                               tunit_hdif=c.hdif_tunit, ddragv=c.ddragv, ddragd=c.ddragd,
                               ddragt=c.ddragt, ddragq=c.ddragq, tunit_damp=c.damp_tunit,
                               ray0=c.ray0, sponge=c.sponge)
        self.semi = SemiImplicit(self.sp, self.vg, self.damping)
        self.vdiff = VerticalDiffusion(self.vg, c.vdifv, c.vdifd, c.vdift, c.vdifq)
        self.integ = Integrator(self.sp, self.vg, self.damping, self.semi, self.vdiff)
        self.batched = getattr(spectral, "batched", False) or self.cfg.nmem > 1
        self.nmem = max(self.cfg.nmem, 1)
        dev = self.sp.device
        if self.batched:
            mk = lambda: State.zeros_ensemble(basic_state.ps, self.vg.kmax, self.nmem,  # noqa
                                              device=dev)
        else:
            mk = lambda: State.zeros(basic_state.ps, self.vg.kmax, device=dev)   # noqa: E731
        self.ga = mk()
        self.gb = mk()
        self.gc = mk()
        self.time = 0.0
        self.istep = 0
        self._stepper = None
        self._last_top = None
        self.phases = None
        self._phase_t = None

    @property
    def device(self):
        return device_name()

    def set_initial_perturbation(self, u=None, v=None, t=None, q=None, ps=None):
        for name, val in (("u", u), ("v", v), ("t", t), ("q", q), ("ps", ps)):
            if val is not None:
                arr = torch.as_tensor(np.asarray(val) if not isinstance(val, torch.Tensor)
                                      else val, dtype=torch.float64).to(self.sp.device)
                setattr(self.ga, name, arr.clone())
                setattr(self.gb, name, arr.clone())

    # ------------------------------------------------------------------
    def diagnostics(self):
        """The eight history fields in grid space (model.py:151-166)."""
        sp, vg = self.sp, self.vg
        if not self.dyn.diag:
            # after a fused run: the diagnostic fields of the top of the last
            # step, as the reference's loop leaves them (model.py:235)
            st = self.ga
            if self._last_top is not None:
                a = self._last_top
                if not self.batched:
                    a = {k: v[0] for k, v in a.items()}
                st = self.ga.copy()
                st.load_spectral(self.sp, a)
            self.dyn.tendencies(st)
        d = self.dyn.diag
        psi = sp.wave_to_grid(sp.inverse_laplacian(d["vor_s"]))
        chi = sp.wave_to_grid(sp.inverse_laplacian(d["div_s"]))
        z = vg.hydrostatic(self.ga.t) / GRAV
        return {"psi": psi, "chi": chi, "u": self.ga.u, "v": self.ga.v, "w": d["omega"],
                "t": self.ga.t, "z": z, "p": self.ga.ps}

    # ------------------------------------------------------------------
    def _forcing_args(self, mjo_forcing, sf):
        frc_t = None
        if mjo_forcing is not None:
            frc_t = mjo_forcing.step()
        elif sf is not None:
            frc_t = sf.t
        return frc_t

    def _general_step(self, dt, start, frc_t, sf, writer_state=None):
        """One reference step on the grid state (model.py:232-243)."""
        frc_vor = sf.vor if sf is not None else None
        frc_div = sf.div if sf is not None else None
        frc_ps = sf.ps if sf is not None else None
        tend = self.dyn.tendencies(self.ga, frc_t=frc_t, frc_vor=frc_vor, frc_div=frc_div,
                                   frc_ps=frc_ps)
        cur_top = self.diagnostics() if writer_state is not None else None
        prev = self.gb.to_spectral(self.sp)
        new = self.integ.step(dt, prev, tend)
        self.gc.load_spectral(self.sp, new)
        if start:
            self.gb.assign(self.ga)
        else:
            self.gb.robert_asselin(self.ga, self.gc, self.cfg.robert)
        self.ga.assign(self.gc)
        return new, cur_top

    def _schedule(self, nsteps):
        """[(dt, is_start)] for the calls of one run (model.py:213-219)."""
        c = self.cfg
        out = []
        istep = 0
        advanced = 0
        while advanced < nsteps:
            istep += 1
            if istep > c.inistp:
                out.append((c.delt, False))
                advanced += 1
            else:
                out.append((c.delt / (2.0 ** (c.inistp - istep + 1)), True))
        return out

    def run(self, mjo_forcing=None, steady_forcing=None, writer=None, verbose=True,
            progress_every=240):
        """Integrate forward; returns self (model.py:169-290)."""
        cfg = self.cfg
        spd = cfg.steps_per_day
        nsteps = int(round(cfg.ndays * spd))
        t0 = _time.time()
        if verbose:
            print(f"  backend: {self.device}", flush=True)
        sched = self._schedule(nsteps)
        self.phases = {} if cfg.phase_timing else None
        if self.phases is not None:
            torch.cuda.synchronize()
            self._phase_t = _time.perf_counter()
        nonzero = any(bool((getattr(st, k) != 0).any()) for st in (self.ga, self.gb)
                      for k in ("u", "v", "t", "q", "ps"))
        if cfg.fused and (writer is None or not nonzero):
            self._run_fused(sched, mjo_forcing, steady_forcing, verbose, progress_every, t0,
                            writer=writer, nonzero=nonzero)
        else:
            self._run_general(sched, mjo_forcing, steady_forcing, writer, verbose,
                              progress_every, t0)
        if verbose:
            print(f"  done: {nsteps} steps, {_time.time() - t0:.1f}s")
        if writer is not None:
            writer.close()
        return self

    # ---- general loop ------------------------------------------------------
    def _run_general(self, sched, mjo_forcing, sf, writer, verbose, progress_every, t0):
        cfg = self.cfg
        spd = cfg.steps_per_day
        out_every = int(round(cfg.out_interval_days * spd))
        acc, nacc, day_done, prev_top = None, 0, 0, None
        advanced = 0
        for istep, (dt, start) in enumerate(sched, 1):
            frc_t = self._forcing_args(mjo_forcing, sf)
            _, cur_top = self._general_step(dt, start, frc_t, sf,
                                            writer_state=True if writer is not None else None)
            if not self.ga.isfinite():
                raise FloatingPointError(
                    f"model blew up at step {istep} (t={self.time / 86400:.2f} d)")
            if start:
                prev_top = cur_top
                continue
            self.time += dt
            advanced += 1
            if writer is not None:
                if prev_top is None:
                    prev_top = cur_top
                fields = {k: 0.5 * (cur_top[k] + prev_top[k]) for k in cur_top}
                if cfg.time_average:
                    if acc is None:
                        acc = {k: torch.zeros_like(v) for k, v in fields.items()}
                    for k, v in fields.items():
                        acc[k] += v
                    nacc += 1
                if advanced % out_every == 0:
                    day_done += 1
                    if cfg.time_average:
                        _emit(writer, day_done, {k: v / nacc for k, v in acc.items()})
                        acc, nacc = None, 0
                    else:
                        _emit(writer, day_done, fields)
            prev_top = cur_top
            if verbose and progress_every and advanced % progress_every == 0:
                self._progress(t0)

    def _progress(self, t0):
        m = self.ga.max_abs()
        print(f"  day {self.time / 86400:6.2f}  |u|max {m['u']:7.3f}  |T|max {m['t']:6.3f}  "
              f"|ps|max {m['ps']:7.4f}   [{_time.time() - t0:5.1f}s]", flush=True)

    # ---- fused loop ----------------------------------------------------------
    def stepper(self):
        if self._stepper is None:
            from .stepper import EnsembleStepper
            self._stepper = EnsembleStepper(
                self.sp, self.vg, self.bst, self.damping, self.semi, self.vdiff, self.nmem,
                precision=self.cfg.precision, robert=self.cfg.robert,
                strictly_linear=self.cfg.strictly_linear,
                tc_off=None if self.cfg.tc_off < 0 else self.cfg.tc_off)
        return self._stepper

    def _state_spectral(self, st):
        spec = st.to_spectral(self.sp)
        if not self.batched:
            spec = {k: v.unsqueeze(0) for k, v in spec.items()}
        return spec

    def _load_stepper(self, stp):
        a = self._state_spectral(self.ga)
        b = self._state_spectral(self.gb)
        stp.load(a, b, self.ga.ps, self.gb.ps)

    def _unload_stepper(self, stp):
        stp.flush()
        if stp.precision != "fp64":
            # FP32 state: the grid levels from the stepper's own synthesis
            # kernels (previous level first: the current one leaves the
            # stepper primed)
            gb = stp.grid_level("b")
            ga = stp.grid_level("a")
            psa, psb = stp.psa.to(torch.float64), stp.psb.to(torch.float64)
            if not self.batched:
                ga = {k: v[0] for k, v in ga.items()}
                gb = {k: v[0] for k, v in gb.items()}
                psa, psb = psa[0], psb[0]
            for st, g, ps in ((self.ga, ga, psa), (self.gb, gb, psb)):
                st.u, st.v, st.t, st.q = g["u"], g["v"], g["t"], g["q"]
                st.ps = ps.clone()
            self.dyn.diag = {}
            return
        a, b = stp.spectral_state()
        if not self.batched:
            a = {k: v[0] for k, v in a.items()}
            b = {k: v[0] for k, v in b.items()}
        psa = stp.psa.to(torch.float64)
        psb = stp.psb.to(torch.float64)
        if not self.batched:
            psa, psb = psa[0], psb[0]
        b_full = dict(b)
        b_full["pi"] = a["pi"]               # placeholder; ps comes from the grid copy
        self.ga.load_spectral(self.sp, a)
        self.ga.ps = psa.clone()
        self.gb.load_spectral(self.sp, b_full)
        self.gb.ps = psb.clone()
        self.dyn.diag = {}

    def _spec_forcing(self, x, is3d):
        """Grid forcing -> spectral with an explicit member axis (B, M, M[, K]),
        B = 1 for a field shared by all members."""
        if x is None:
            return None
        sp = self.sp
        t = x.to(sp.device) if isinstance(x, torch.Tensor) else torch.as_tensor(
            np.asarray(x), device=sp.device)
        t = t.to(torch.float64)
        K = self.vg.kmax if is3d else 1
        g4 = t.reshape((-1, sp.nlat, sp.nlon, K)).contiguous()
        s = sp._anal(sp._fwd(g4), sp._t["Pgw"], 0)
        return s if is3d else s[..., 0]

    def _diagnostics_mean(self, spec, ps):
        """The eight history fields of a mean spectral state and mean grid ps'
        (the reference's diagnostics, model.py:151-166, are linear in both, so
        this equals the mean of the per-step fields)."""
        sp, vg = self.sp, self.vg
        if not self.batched:
            spec = {k: v[0] for k, v in spec.items()}
            ps = ps[0]
        u, v = sp.vordiv_to_uv(spec["vor"], spec["div"])
        t = sp.wave_to_grid(spec["t"])
        q = sp.wave_to_grid(spec["q"])
        vor = sp.wave_to_grid(spec["vor"])
        div = sp.wave_to_grid(spec["div"])
        pix, piy = sp.hgrad(spec["pi"])
        st = types.SimpleNamespace(u=u, v=v, t=t, q=q, ps=ps)
        o = self.dyn._grid_kernel(st, vor, div, pix, piy, None, None, None)
        psi = sp.wave_to_grid(sp.inverse_laplacian(spec["vor"]))
        chi = sp.wave_to_grid(sp.inverse_laplacian(spec["div"]))
        z = vg.hydrostatic(t) / GRAV
        return {"psi": psi, "chi": chi, "u": u, "v": v, "w": o["omega"], "t": t, "z": z,
                "p": ps}

    def _mark(self, name):
        """Add the seconds since the previous mark to phase `name` (only with
        Config.phase_timing; the device is synchronised first so that the
        phase's GPU work is counted in it)."""
        if self.phases is None:
            return
        torch.cuda.synchronize()
        now = _time.perf_counter()
        self.phases[name] = self.phases.get(name, 0.0) + (now - self._phase_t)
        self._phase_t = now

    def _blew_up(self, stp, a, b):
        """FloatingPointError of the fused loop (model.py:245-247 raises at the
        step itself): the device flags are read at day boundaries and at the
        end of a run, so the message names the window of calls since the last
        clean check and the members whose flags are set."""
        bad = stp.bad_members()
        who = (f"member{'s' if len(bad) > 1 else ''} {', '.join(map(str, bad))}"
               if self.batched else "the model")
        raise FloatingPointError(
            f"model blew up at a step between {a + 1} and {b} of this run "
            f"(t <= {self.time / 86400:.2f} d): non-finite values in {who}")

    def _run_fused(self, sched, mjo_forcing, sf, verbose, progress_every, t0, writer=None,
                   nonzero=True):
        cfg = self.cfg
        stp = self.stepper()
        stp.set_timesteps(sorted({dt for dt, _ in sched}))
        fv = self._spec_forcing(sf.vor, True) if sf is not None else None
        fd = self._spec_forcing(sf.div, True) if sf is not None else None
        fp = self._spec_forcing(sf.ps, False) if sf is not None else None
        ft_steady = (self._spec_forcing(sf.t, True)
                     if (sf is not None and mjo_forcing is None) else None)
        last_src = [None]

        def install(ft):
            xs = (fv, fd, ft, fp)
            per = any(x is not None and x.shape[0] > 1 for x in xs)
            stp.set_forcing(frc_vor=fv, frc_div=fd, frc_t=ft, frc_pi=fp, per_member=per)

        first = 0
        if nonzero:
            # forward start from an arbitrary grid state: one general step
            dt, start = sched[0]
            frc_t = self._forcing_args(mjo_forcing, sf)
            last_src[0] = frc_t if mjo_forcing is not None else None
            self._general_step(dt, start, frc_t, sf)
            first = 1
            if not start:
                self.time += dt
        if mjo_forcing is None:
            install(ft_steady)
        # a forcing of daily records (MJOForcing): records analysed once, each
        # step's forcing interpolated in spectral space on the device
        interp = None
        if mjo_forcing is not None and SpectralInterpolation.supports(mjo_forcing):
            interp = SpectralInterpolation(mjo_forcing, lambda g: self._spec_forcing(g, True))

        def next_forcing():
            src = interp.next() if interp is not None else mjo_forcing.step()
            if src is not last_src[0]:
                last_src[0] = src
                self._mark("steps")
                install(src if interp is not None else self._spec_forcing(src, True))
                self._mark("forcing")

        self._last_top = None
        advanced = 1 if (first == 1 and not sched[0][1]) else 0
        if first >= len(sched):
            return
        self._mark("setup")
        if nonzero or first:
            self._load_stepper(stp)
        else:
            stp.load_zero()          # a zero state is zero in every representation
        self._mark("load")
        spd = cfg.steps_per_day
        out_every = int(round(cfg.out_interval_days * spd))
        day_done, sampled = 0, False
        if writer is not None:
            stp.hist_begin()
        i = first
        checked = first          # calls of this run known to be finite
        while i < len(sched):
            if writer is not None:
                # history: one step per call, sampled around its kernels
                dt, start = sched[i]
                if mjo_forcing is not None:
                    next_forcing()
                mode = 0 if start else 1
                if i == len(sched) - 1:
                    self._last_top = stp.snapshot()
                if mode == 1 and not sampled:
                    stp.hist_sample("spec", 0)           # no earlier top: prev = cur
                if mode == 1 and not cfg.time_average:
                    stp.hist_reset()
                stp.hist_sample("spec", mode)
                stp.run([(dt, start)], use_graph=False)
                if mode == 1 and not sampled:
                    stp.hist_sample("ps", 0)
                stp.hist_sample("ps", mode)
                sampled = True
                i += 1
                if not start:
                    self.time += dt
                    advanced += 1
                # the blow-up check comes before the day's record is written,
                # as in the reference's loop (model.py:245-277)
                if (not start and advanced % spd == 0) or i == len(sched):
                    if not stp.check_finite():
                        self._blew_up(stp, checked, i)
                    checked = i
                if not start and advanced % out_every == 0:
                    day_done += 1
                    fields = self._diagnostics_mean(*stp.hist_mean())
                    _emit(writer, day_done, fields)
                    stp.hist_reset()
                continue
            if mjo_forcing is not None:
                # time-varying forcing: one .step() call per model step
                next_forcing()
                j = i + 1
            else:
                j, n_adv = i, 0
                while j < len(sched) and (sched[j][1] or n_adv < spd):
                    n_adv += 0 if sched[j][1] else 1
                    j += 1
            chunk = sched[i:j]
            if j == len(sched):
                if len(chunk) > 1:
                    stp.run(chunk[:-1], use_graph=cfg.use_graph)
                self._last_top = stp.snapshot()
                stp.run(chunk[-1:], use_graph=False)
            else:
                stp.run(chunk, use_graph=cfg.use_graph and mjo_forcing is None)
            i = j
            for dt, start in chunk:
                if not start:
                    self.time += dt
                    advanced += 1
            if i == len(sched) or (advanced and advanced % spd == 0):
                if not stp.check_finite():
                    self._blew_up(stp, checked, i)
                checked = i
            if (verbose and progress_every and advanced and advanced % progress_every == 0
                    and i < len(sched)):
                self._unload_stepper(stp)
                self._progress(t0)
        self._mark("steps")
        self._unload_stepper(stp)
        self._mark("unload")

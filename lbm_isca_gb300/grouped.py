"""Ensembles of uneven truncations and level counts stepped together.

The reference batches members of one grid only (ensemble.py:41-106: every
member shares the Spectral and VerticalGrid of the batch).  A
``GroupedEnsemble`` holds one fused stepper per group -- e.g. 48 members at
T21L20, 32 at T42L20 and 16 at T85L40 -- and advances all groups together:
the start-up calls per group, then every stretch of identical steady steps
as ONE CUDA graph whose branches are the groups' step kernels on their own
streams, so one graph launch advances every member of every truncation and
the groups' kernels overlap on the GPU.  Each group's tensor-core tile
choice comes from the autotuner (``autotune.tune``) when the precision uses
the tensor cores.  Every group's result equals that group run alone (same
kernels, same order on its own state).
"""

from __future__ import annotations

import torch

from . import autotune
from .ensemble import EnsembleForcing, make_ensemble_model
from .model import Config


class GroupedEnsemble:
    """groups: list of dicts with nlon, nlat, nmax, sigm (K + 1 half levels),
    basic_state, heats [E][J][I][K] (K/s), and optionally precision and
    config (Config keywords of that group, over the shared ones); config:
    Config keywords shared by every group."""

    def __init__(self, groups, config=None, precision="bf16x3", tune=True, graph_chunk=72):
        self.groups = []
        self.graph_chunk = int(graph_chunk)
        for g in groups:
            kw = dict(config or {})
            kw.update(g.get("config", {}))
            kw["precision"] = g.get("precision", precision)
            m, sp, vg = make_ensemble_model(g["basic_state"], len(g["heats"]), Config(**kw),
                                            device="gb300", nlon=g["nlon"], nlat=g["nlat"],
                                            nmax=g["nmax"], sigm=g["sigm"])
            stp = m.stepper()
            rec = autotune.tune(stp) if tune else None
            self.groups.append({"model": m, "stepper": stp, "heats": g["heats"],
                                "tile": rec})
        self._graphs = {}
        self._cap = torch.cuda.Stream()

    @property
    def members(self):
        return sum(g["stepper"].E for g in self.groups)

    def load(self, nsteps):
        """Zero state, each group's forcing installed, operators for the
        schedule of `nsteps` advancing steps."""
        self.scheds = []
        for g in self.groups:
            m, stp = g["model"], g["stepper"]
            sched = m._schedule(nsteps)
            stp.set_timesteps(sorted({dt for dt, _ in sched}))
            frc = EnsembleForcing(g["heats"], device="gb300").step()
            stp.set_forcing(frc_t=m._spec_forcing(frc, True), per_member=True)
            stp.load_zero()
            self.scheds.append(sched)

    def _graph(self, n):
        """One CUDA graph of n steady steps of every group, each group's step
        kernels on its own stream (captured from the library's stepper
        operator)."""
        # a graph holds the steppers' buffer addresses: it is reused while no
        # stepper has rebuilt its descriptor (which happens when a buffer changes)
        for grp in self.groups:
            grp["stepper"].desc()
        key = (n,) + tuple(grp["stepper"].desc_gen for grp in self.groups)
        g = self._graphs.get(key)
        if g is not None:
            return g
        graph = torch.cuda.CUDAGraph()
        cap = self._cap
        cap.wait_stream(torch.cuda.current_stream())
        for grp in self.groups:
            stp = grp["stepper"]
            cap.wait_stream(stp.stream)
        with torch.cuda.graph(graph, stream=cap):
            for grp in self.groups:
                stp = grp["stepper"]
                dt = stp._dts[-1]
                stp.stream.wait_stream(cap)
                with torch.cuda.stream(stp.stream):
                    torch.ops.lbm_gb300.stepper_run(*stp.op_args(), [dt] * n,
                                                    [stp.set_index(dt)] * n, [2] * n, [1] * n)
                cap.wait_stream(stp.stream)
        self._graphs[key] = graph
        return graph

    def run(self, nsteps):
        """Advance every group by `nsteps` advancing steps after its start-up
        calls (the reference's schedule, model.py:213-219)."""
        self.load(nsteps)
        # start-up calls and the first steady step (whose ps update differs)
        for grp, sched in zip(self.groups, self.scheds):
            stp = grp["stepper"]
            n0 = grp["model"].cfg.inistp + 1
            stp.run(sched[:n0], use_graph=False)
        left = nsteps - 1
        for grp in self.groups:
            torch.cuda.current_stream().wait_stream(grp["stepper"].stream)
        while left > 0:
            n = min(left, self.graph_chunk)
            self._graph(n).replay()
            left -= n
        for grp in self.groups:
            grp["stepper"].stream.wait_stream(torch.cuda.current_stream())
            grp["stepper"].pending_ps_mode = 2
        return self

    def check_finite(self):
        return all(g["stepper"].check_finite() for g in self.groups)

    def spectral_states(self):
        """Per group: the current level (rectangle dicts, member axis first)."""
        return [g["stepper"].spectral_state()[0] for g in self.groups]

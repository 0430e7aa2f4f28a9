#!/usr/bin/env python3
"""Benchmark of the GB300 dynamical-core hot path.

Metric: T42L20 member-steps/s of the batched ensemble (512 members, FP32
state, seeded heatings, plain damping) through the fused stepper; a "step"
is one semi-implicit leapfrog step of every member.  The synthetic workload
is defined in lbm_isca_gb300/configs.py (no dataset is involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun each rank integrates its own
512 members (weak scaling, no collective in the step); the timed region is
bracketed by a barrier and device synchronisation and the max over ranks is
reported.  `--impl reference` times the CPU reference algorithm (the numpy
oracle restatement, oracle/lbm_oracle.py) on this host's cores.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import signal
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "T42L20 member-steps/s, batched mixed-prec vs plain FP64 at <=1e-5 rel L2 err"
UNIT = "member-steps/s"
GRID = (128, 64, 42)
K_LEV = 20
SEED = 1
DTYPES = {"fp32": "f32", "fp64": "f64", "bf16x3": "bf16x3 split, f32 accumulate",
          "bf16split": "bf16x2 split, f32 accumulate"}
SPLIT_NOTE = {"bf16x3": "tcgen05, bf16 3-way split, 6 products, FP32 accumulate",
              "bf16split": "tcgen05, bf16 2-way split, 3 products, FP32 accumulate"}


def placement(stp):
    """Where the step's contractions run, from the stepper's own choice."""
    if stp.precision == "fp64":
        return "all contractions in FP64"
    if not stp.legendre:
        return "all contractions on the FP32 FMA pipes"
    on = {"Legendre analysis": not (stp.tc_off & 1), "Legendre synthesis": not (stp.tc_off & 2),
          "longitude analysis of the level rows": (stp.tc_dft is not None
                                                   and not (stp.tc_off & 4))}
    tc = [k for k, v in on.items() if v]
    fma = [k for k, v in on.items() if not v] + ["longitude synthesis", "surface rows"]
    return (f"{', '.join(tc) or 'nothing'} on the tensor cores ({SPLIT_NOTE[stp.precision]}); "
            f"{', '.join(fma)} on the FP32 FMA pipes")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=720)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--members", type=int, default=512)
    ap.add_argument("--precision", default="bf16x3",
                    choices=["fp32", "fp64", "bf16x3", "bf16split"])
    ap.add_argument("--tc-off", type=int, default=-1,
                    help="bf16 modes: contractions kept on the FMA pipes (bit 0 Legendre "
                         "analysis, 1 Legendre synthesis, 2 longitude analysis; -1: the "
                         "precision's default)")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the accuracy / plain-FP64 / CPU side measurements")
    ap.add_argument("--adjoint", action="store_true",
                    help="checkpointed-adjoint cost and accuracy (T42L20, 20 days, FP64, "
                         "every state stored; 32 on the binomial schedule for comparison) "
                         "instead of the bench")
    ap.add_argument("--adjoint-precision", default="fp64", choices=["fp64", "fp32"],
                    help="--adjoint: working precision of the adjoint and its forward runs")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="--adjoint over this many steps instead of 20 days (profiling)")
    ap.add_argument("--adjoint-members", type=int, default=None,
                    help="--adjoint: time one gradient of this many members (own heatings) "
                         "against one single-member gradient instead")
    ap.add_argument("--fd-dirs", type=int, default=16,
                    help="central-difference directions checked by --adjoint")
    ap.add_argument("--cpu-plans", action="store_true",
                    help="CPU baselines on the host: one member with all BLAS threads "
                         "(T42L20, T85L40) and the oracle batched over 512 members, "
                         "instead of the bench")
    ap.add_argument("--conditioning", action="store_true",
                    help="conditioning of the 30-day problem: FP64 against FP64 with the "
                         "heatings rounded to FP32, and with the day-10 state kicked by one "
                         "FP32-sized relative change, next to FP32 and bf16x3 against FP64; "
                         "the bench's 512-member T42L20 ensemble, T42L20 x 128 and T85L40 x 8 "
                         "strictly linear; instead of the bench")
    ap.add_argument("--uneven-groups-adjoint", action="store_true",
                    help="--uneven-groups: then each group's gradient of the area-mean "
                         "streamfunction response (sigma 0.25, 30-60N 150-210E; precision "
                         "from --adjoint-precision)")
    ap.add_argument("--uneven-groups", action="store_true",
                    help="uneven batching: 48 T21L20 + 32 T42L20 + 16 T85L40 members (seed 4, "
                         "strictly linear), 20 days in one CUDA graph per stretch of steady "
                         "steps, autotuned tensor-core tiles per truncation, instead of the "
                         "bench")
    ap.add_argument("--sweep", action="store_true",
                    help="precision sweep (fp32, bf16x3 and bf16split against FP64 per field "
                         "at days 10 and 30, T42L20 x 128 members and T85L40 x 8 members) "
                         "instead of the bench")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# CPU side: the oracle (reference algorithm) on the host cores
# ---------------------------------------------------------------------------
def _oracle_worker(args):
    """One single-member T42L20 oracle run; returns (steps, seconds)."""
    member, warm, budget_s, max_steps = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from oracle import lbm_oracle as orc
    from lbm_isca_gb300 import configs
    nlon, nlat, nmax = GRID
    sigm = configs.equal_sigma_half_levels(K_LEV)
    heats, _ = configs.ensemble_heating(nlon, nlat, sigm, member + 1, seed=SEED)
    tr = orc.SphericalTransform(nlon, nlat, nmax)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(nlon, nlat, sigm)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(K_LEV)))
    frc = heats[member]
    for _ in range(warm):
        m.step(frc_t=frc)
    t0 = time.perf_counter()
    n = 0
    while n < max_steps and (time.perf_counter() - t0) < budget_s:
        m.step(frc_t=frc)
        n += 1
    return n, time.perf_counter() - t0


def cpu_oracle_throughput(nproc, warm, budget_s, max_steps=10 ** 9):
    """member-steps/s of `nproc` concurrent single-thread oracle runs."""
    ctx = mp.get_context("spawn")
    env_keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in env_keys}
    for k in env_keys:
        os.environ[k] = "1"
    try:
        with ctx.Pool(nproc) as pool:
            res = pool.map(_oracle_worker, [(e, warm, budget_s, max_steps)
                                            for e in range(nproc)])
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    rate = sum(n / s for n, s in res)
    return rate, res


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def mem_available_bytes():
    """MemAvailable of the host (Linux), or None."""
    try:
        with open("/proc/meminfo") as fh:
            for line in fh:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def cpu_plans(budget_s=30.0, bytes_per_member=50e6):
    """The CPU baselines besides the one-member-per-core throughput: (i) one
    member with the BLAS threads on all host cores (numpy's default in this
    process) at T42L20 and T85L40; (iii) the oracle batched over up to 512
    members (its member axis, as make_ensemble_model(device="cpu") batches)
    at T42L20, as many as fit in 30% of the host's available memory at
    about `bytes_per_member` each (45 MB measured peak); each after one
    warm-up step, timed over as many steps as fit in `budget_s` (at least
    one)."""
    from oracle import lbm_oracle as orc
    from lbm_isca_gb300 import configs
    avail = mem_available_bytes()
    e_big = 512 if avail is None else max(1, min(512, int(0.3 * avail / bytes_per_member)))
    out = {"cores": host_cores(), "mem_available_gb": None if avail is None else avail / 1e9}

    def timed_steps(m, frc):
        m.step(frc_t=frc)
        t0 = time.perf_counter()
        n = 0
        while n == 0 or (time.perf_counter() - t0) < budget_s:
            m.step(frc_t=frc)
            n += 1
        return n, time.perf_counter() - t0

    for label, (nlon, nlat, nmax, K, E) in (("single_T42L20", (128, 64, 42, 20, None)),
                                            ("single_T85L40", (256, 128, 85, 40, None)),
                                            ("batched_T42L20", (128, 64, 42, 20, e_big))):
        sigm = configs.equal_sigma_half_levels(K)
        tr = orc.SphericalTransform(nlon, nlat, nmax)
        lv = orc.SigmaLevels(sigm)
        bs = configs.solid_body_basic_state(nlon, nlat, sigm)
        heats, _ = configs.ensemble_heating(nlon, nlat, sigm, E or 1, seed=SEED)
        m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(K)), nmem=E)
        n, sec = timed_steps(m, heats if E else heats[0])
        out[label] = {"members": E or 1, "steps": n, "seconds": sec,
                      "ms_per_step": 1000.0 * sec / n,
                      "member_steps_per_s": (E or 1) * n / sec}
        print(json.dumps({"cpu_plan": {label: out[label]}}), file=sys.stderr, flush=True)
        del m
    return out


def reference_arm(args):
    """`--impl reference`: the reference algorithm on the host cores."""
    cores = min(host_cores(), 64)
    # each worker: W warm-up steps, then up to K steps (bounded in time)
    budget = max(5.0, min(120.0, args.cpu_seconds * 4))
    rate, res = cpu_oracle_throughput(cores, max(1, min(args.warmup, 3)), budget,
                                      max_steps=args.steps)
    steps = int(min(n for n, _ in res))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * cores / rate if rate else None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "T42L20 solid-body basic state, seeded elliptic heatings "
                               "(seed 1), plain damping; one member per host process",
                   "members": cores, "grid": "T42 128x64", "levels": 20},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} concurrent single-thread numpy oracle runs, "
                                   f"{steps}+ steps each"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True,
                start_new_session=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            try:
                os.killpg(self.proc.pid, signal.SIGTERM)
            except Exception:
                pass
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r)
                          if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def build_model(E, precision, torch, days=1.0, seed=SEED, device="cuda"):
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.ensemble import make_ensemble_model
    from lbm_isca_gb300.model import Config
    nlon, nlat, nmax = GRID
    sigm = configs.equal_sigma_half_levels(K_LEV)
    bs = configs.solid_body_basic_state(nlon, nlat, sigm)
    cfg = Config(ndays=days, precision=precision, tc_off=TC_OFF,
                 **configs.plain_damping(K_LEV))
    model, spb, vg = make_ensemble_model(bs, E, cfg, device=device, nlon=nlon, nlat=nlat,
                                         nmax=nmax, sigm=sigm)
    heats, _ = configs.ensemble_heating(nlon, nlat, sigm, E, seed=seed)
    return model, heats


def step_roofline(E, p, ms_per_step, peaks, precision):
    """The whole step against its lower bound, with the per-member-step counts
    of the reference algorithm: Legendre flops 4 NS J (33 K + 6), DFT flops
    (21 K + 6) J 2.5 I log2 I, unavoidable HBM bytes = the state read and
    written (4 (4 K + 1) NS 2 p) plus the grid forcing (K J I p).  T_min =
    transform flops / contraction peak + unavoidable bytes / HBM peak; the
    contraction peak is the measured bf16 tensor rate for the tensor-core
    modes and the FP32 FMA rate (152 SMs x 128 lanes x 2 x max clock) for the
    FMA path."""
    nlon, nlat, nmax = GRID
    J, I, K = nlat, nlon, K_LEV
    NS = (nmax + 1) * (nmax + 2) // 2
    leg = 4.0 * NS * J * (33 * K + 6)
    dft = (21 * K + 6) * J * 2.5 * I * math.log2(I)
    byt = 4.0 * (4 * K + 1) * NS * 2 * p + K * J * I * p
    hbm = float(peaks.get("hbm_gbs", 6800.0)) * 1e9
    if precision in ("bf16x3", "bf16split"):
        pk, pk_name = float(peaks.get("bf16_tflops", 1900.0)) * 1e12, "bf16 tensor (measured)"
    else:
        mhz = float(peaks.get("sm_max_mhz", 2070.0))
        pk, pk_name = 152 * 128 * 2 * mhz * 1e6, "FP32 FMA (152 SMs x 128 x 2 x max clock)"
    t_min = E * (leg + dft) / pk + E * byt / hbm
    return {"t_min_ms": 1e3 * t_min, "t_measured_ms": ms_per_step,
            "frac": 1e3 * t_min / ms_per_step,
            "per_member_step": {"legendre_flop": leg, "dft_flop": dft, "unavoidable_bytes": byt},
            "contraction_peak": pk_name}


def algorithmic_bytes(E, p):
    """HBM bytes each stepper kernel must move per launch (p = bytes/real):
    every array it reads or writes once, per-member arrays times E, the shared
    basic state once."""
    nlon, nlat, nmax = GRID
    M, J, I, K = nmax + 1, nlat, nlon, K_LEV
    NS = M * (M + 1) // 2
    c = 2 * p
    shared_grid = p * (14 * J * K * I + J * (K + 1) * I + 5 * J * I)
    sf = c * M * J * (6 * K + 5)
    af = c * M * J * (7 * K + 2)
    g6 = 4 * J * I * (6 + 6 * K)
    g9 = 4 * J * I * (2 + 9 * K)
    st3 = c * 4 * NS * K
    out = {
        "anal": E * (af + c * (4 * NS * K + 2 * NS)),
        "implicit": E * (3 * st3 + c * 2 * NS + 2 * st3 + c * 4 * NS),
        "synth": E * (st3 + c * 4 * NS + sf),
    }
    if p == 4:      # FP32: the grid-point part is three launches
        out.update({"idft": E * (sf + g6),
                    "alg": E * (g6 + g9 + 4 * p * J * I) + shared_grid,
                    "fdft": E * (g9 + af)})
    else:
        out["grid"] = E * (sf + af + 4 * p * J * I) + shared_grid
    return out


def traffic_key(stp, name):
    """Record name of a step kernel in the traffic file: `name`, or
    `name`_tc when that contraction runs on the tensor cores."""
    tc = stp.legendre and {"anal": not (stp.tc_off & 1), "synth": not (stp.tc_off & 2),
                           "fdft": stp.tc_dft is not None and not (stp.tc_off & 4)}.get(name)
    return name + "_tc" if tc else name


def read_traffic(kernel, E):
    """DRAM bytes per launch of `kernel` from the committed ncu record
    (profiles/dram_traffic_t42l20.json), scaled from its member count to E
    (the traffic of every stepper kernel grows in proportion to the members)."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_t42l20.json")
    try:
        rec = json.load(open(path))
        return float(rec["bytes_per_launch"][kernel]) * E / float(rec["members"])
    except Exception:
        return None


def precision_sweep(torch, days=(10, 30),
                    precisions=("fp32", "bf16x3", "bf16split")):
    """Each working precision against FP64 (which equals the oracle to
    1e-10) per prognostic field at days 10 and 30, on seeded ensemble
    heatings (seed 2): T42L20 with 128 members (dt 1200 s) with the
    reference's default dynamics (its kinetic-energy term keeps the nonlinear
    0.5 |v'|^2) and strictly linear, T85L40 with 8 members (dt 600 s)
    strictly linear (with the default dynamics strongly forced T85L40
    members grow without bound by day 14, FP64 included).  One run per
    precision to day 30 through the fused stepper, the state taken at the end
    of day 10 and of day 30; relative L2 over all members per field, and per
    member (worst field) the median, the maximum and the shares within 1e-5
    and 1e-3.  Each case is printed as it completes."""
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.ensemble import make_ensemble_model
    from lbm_isca_gb300.model import Config
    out = {}
    cases = [("T42L20_default", 128, 64, 42, 20, 128, 1200.0, False),
             ("T42L20_strictly_linear", 128, 64, 42, 20, 128, 1200.0, True),
             ("T85L40_strictly_linear", 256, 128, 85, 40, 8, 600.0, True)]
    for (label, nlon, nlat, nmax, K, E, delt, lin) in cases:
        sigm = configs.equal_sigma_half_levels(K)
        bs = configs.solid_body_basic_state(nlon, nlat, sigm)
        heats, _ = configs.ensemble_heating(nlon, nlat, sigm, E, seed=2)
        spd = int(round(86400.0 / delt))
        runs, secs = {}, {}
        for prec in ("fp64",) + tuple(precisions):
            cfg = Config(ndays=max(days), precision=prec,
                         **dict(configs.plain_damping(K), delt=delt, strictly_linear=lin))
            m, _, _ = make_ensemble_model(bs, E, cfg, device="cuda", nlon=nlon, nlat=nlat,
                                          nmax=nmax, sigm=sigm)
            stp = m.stepper()
            sched = m._schedule(spd * max(days))
            stp.set_timesteps(sorted({dt for dt, _ in sched}))
            stp.set_forcing(frc_t=m._spec_forcing(torch.as_tensor(heats, device="cuda"), True),
                            per_member=True)
            stp.load_zero()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            snaps, done = {}, 0
            for d in sorted(days):
                upto = spd * d + m.cfg.inistp
                stp.run(sched[done:upto], use_graph=True)
                done = upto
                torch.cuda.synchronize()
                # copies: .to() of an FP64 state would return a view of it
                snaps[d] = (None if not stp.check_finite() else
                            {k: x.to(torch.complex128, copy=True) for k, x in
                             (("vor", stp.sa3[:, 0]), ("div", stp.sa3[:, 1]),
                              ("t", stp.sa3[:, 2]), ("pi", stp.sas[:, 0]), ("q", stp.sa3[:, 3]))})
            secs[prec] = time.perf_counter() - t0
            runs[prec] = snaps
            del m, stp
        rec = {"members": E, "dt_s": delt, "strictly_linear": lin, "run_s": secs}
        for prec in precisions:
            for d in sorted(days):
                r, x = runs["fp64"][d], runs[prec][d]
                if r is None or x is None:
                    rec[f"{prec}_day{d}"] = "non-finite"
                    continue
                e, mem = {}, None
                for k in ("vor", "div", "t", "pi"):
                    e[k] = float(torch.linalg.norm(x[k] - r[k]) / torch.linalg.norm(r[k]))
                    dims = tuple(range(1, r[k].dim()))
                    pm = (torch.linalg.vector_norm(x[k] - r[k], dim=dims)
                          / torch.linalg.vector_norm(r[k], dim=dims))
                    mem = pm if mem is None else torch.maximum(mem, pm)
                e["q_absmax"] = float(x["q"].abs().max())
                e["members_within_1e-5"] = float((mem <= 1e-5).double().mean())
                e["members_within_1e-3"] = float((mem <= 1e-3).double().mean())
                e["member_median"] = float(mem.median())
                e["member_max"] = float(mem.max())
                rec[f"{prec}_day{d}"] = e
        out[label] = rec
        print(json.dumps({"precision_sweep_case": {label: rec}}), flush=True)
    return out


def uneven_groups_measurement(torch, precision, days=20, groups=((64, 32, 21, 20, 48),
                                                             (128, 64, 42, 20, 32),
                                                             (256, 128, 85, 40, 16)),
                        adjoint=None):
    """Members of three truncations stepped together (GroupedEnsemble): the
    seeded heatings of every group drawn in order from one generator (seed
    4), solid-body basic states, plain damping, strictly linear dynamics (the
    reference dynamics let strongly forced T85L40 members grow without bound
    by day 14), dt 1200 s, `days` model days; device time of the whole run
    and of the steady part, per-group tile choices of the autotuner, and each
    group's state against the same group run alone (bitwise)."""
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.grouped import GroupedEnsemble
    sig = {K: configs.equal_sigma_half_levels(K) for K in {g[3] for g in groups}}
    heats = configs.grouped_heating([(nlon, nlat, sig[K], E)
                                     for nlon, nlat, _, K, E in groups], seed=4)
    specs = [dict(nlon=nlon, nlat=nlat, nmax=nmax, sigm=sig[K], heats=h,
                  basic_state=configs.solid_body_basic_state(nlon, nlat, sig[K]),
                  config=dict(configs.plain_damping(K), strictly_linear=True))
             for (nlon, nlat, nmax, K, E), h in zip(groups, heats)]
    ge = GroupedEnsemble(specs, precision=precision, tune=True)
    nsteps = 72 * days
    ge.run(4)                                   # capture the graphs, warm up
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    ge.run(nsteps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    finite = ge.check_finite()
    E = ge.members
    out = {"workload": "48 T21L20 + 32 T42L20 + 16 T85L40 members, seeded heatings (seed 4), "
                       f"strictly linear, dt 1200 s, {days} days, {precision}",
           "members": E, "steps": nsteps, "seconds": ms / 1000.0,
           "member_steps_per_s": E * nsteps / (ms / 1000.0), "finite": finite,
           "tiles": [{"grid": f"T{g['stepper'].N}L{g['stepper'].K}",
                      "members": g["stepper"].E, "choice": g["tile"]} for g in ge.groups]}
    if adjoint:
        out["adjoint"] = uneven_groups_adjoint(torch, ge, nsteps, adjoint)
    return out


def uneven_groups_adjoint(torch, ge, nsteps, precision):
    """The adjoint half of the uneven-truncation workload: for each group,
    every member's gradient of its own response (area-mean psi' at sigma 0.25
    over 30-60N 150-210E at the end of the run) with respect to its
    heating, over the same calls as the forward run, by the checkpointed
    adjoint in `precision` (every state stored where the group's trajectory
    fits in half the free HBM, else as many as fit on the binomial schedule);
    each group reversed as one batched model, one group after another (not
    inside the grouped graph).  Seconds of one gradient against one forward
    run of the same calls, member-gradients per second."""
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    res = []
    for g in ge.groups:
        m = g["model"]
        h = torch.as_tensor(g["heats"], device="cuda")

        def make(n, **kw):
            fg = ForcingGradient(m, None, nsteps=n, precision=precision, **kw)
            fg.response = AreaMeanStreamfunction(fg.step.sp, m.vg)
            return fg

        warm = make(4, snaps=2)
        warm.value_and_grad(h)                       # captures every graph variant
        fg = make(nsteps)
        fg._fg, fg._ag = warm._fg, warm._ag
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Jf = fg.value(h)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        J, grad = fg.value_and_grad(h)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        E = int(h.shape[0])
        res.append({"grid": f"T{m.sp.nmax}L{m.vg.kmax}", "members": E,
                    "calls": len(fg.calls), "stored_states": fg.snaps,
                    "forward_steps_in_gradient": fg.forward_steps,
                    "forward_s": t1 - t0, "gradient_s": t2 - t1,
                    "gradient_over_forward": (t2 - t1) / (t1 - t0),
                    "member_gradients_per_s": E / (t2 - t1),
                    "J_forward_equals_gradient_sweep": bool(torch.equal(Jf, J)),
                    "finite": bool(torch.isfinite(grad).all())})
        del warm, fg, grad
        torch.cuda.empty_cache()
    return res


def conditioning(torch, days=(10, 30), kick=1e-7):
    """How much of the FP32-against-FP64 difference the problem itself sets.
    Against the unperturbed FP64 run: (1) the FP64 run with each heating
    rounded to FP32 (every input changed by less than 2^-24 relatively);
    (2) the FP64 run whose state (both levels, spectral and grid ps') is
    multiplied at the end of day 10 by (1 + ``kick`` n), n a seeded standard
    normal per value -- one FP32-sized rounding of the developed state, then
    exact FP64 arithmetic: its day-30 difference over ``kick`` is the growth
    the problem gives to a single rounding error; beside the FP32 (FMA)
    stepper and the bf16x3 stepper.  Relative L2 per field over all members,
    and per member (worst field) the median, maximum and share within 1e-5.
    Cases: the bench's own T42L20 ensemble (512 members, heatings seed 1, the
    reference's dynamics with the kinetic-energy term), T42L20 x 128 members
    strictly linear (seed 2), T85L40 x 8 members strictly linear (seed 2,
    dt 600 s)."""
    from lbm_isca_gb300 import configs
    from lbm_isca_gb300.ensemble import make_ensemble_model
    from lbm_isca_gb300.model import Config
    out = {}
    cases = [("T42L20_bench_ensemble", 128, 64, 42, 20, 512, 1200.0, False, SEED),
             ("T42L20_strictly_linear", 128, 64, 42, 20, 128, 1200.0, True, 2),
             ("T85L40_strictly_linear", 256, 128, 85, 40, 8, 600.0, True, 2)]
    for (label, nlon, nlat, nmax, K, E, delt, lin, seed) in cases:
        sigm = configs.equal_sigma_half_levels(K)
        bs = configs.solid_body_basic_state(nlon, nlat, sigm)
        heats, _ = configs.ensemble_heating(nlon, nlat, sigm, E, seed=seed)
        spd = int(round(86400.0 / delt))
        runs = {}
        for name, prec, h in (("fp64", "fp64", heats),
                              ("fp64_input_rounded", "fp64",
                               heats.astype(np.float32).astype(np.float64)),
                              ("fp64_kicked_day10", "fp64", heats),
                              ("fp32", "fp32", heats), ("bf16x3", "bf16x3", heats)):
            cfg = Config(ndays=max(days), precision=prec,
                         **dict(configs.plain_damping(K), delt=delt, strictly_linear=lin))
            m, _, _ = make_ensemble_model(bs, E, cfg, device="cuda", nlon=nlon, nlat=nlat,
                                          nmax=nmax, sigm=sigm)
            stp = m.stepper()
            sched = m._schedule(spd * max(days))
            stp.set_timesteps(sorted({dt for dt, _ in sched}))
            stp.set_forcing(frc_t=m._spec_forcing(torch.as_tensor(h, device="cuda"), True),
                            per_member=True)
            stp.load_zero()
            snaps, done = {}, 0
            for d in sorted(days):
                upto = spd * d + m.cfg.inistp
                stp.run(sched[done:upto], use_graph=True)
                done = upto
                torch.cuda.synchronize()
                # copies: .to() of an FP64 state would return a view of it
                snaps[d] = (None if not stp.check_finite() else
                            {k: x.to(torch.complex128, copy=True) for k, x in
                             (("vor", stp.sa3[:, 0]), ("div", stp.sa3[:, 1]),
                              ("t", stp.sa3[:, 2]), ("pi", stp.sas[:, 0]))})
                if name == "fp64_kicked_day10" and d == 10:
                    stp.flush()
                    g = torch.Generator(device="cuda").manual_seed(7)
                    for x in (stp.sa3, stp.sb3, stp.sas, stp.psa, stp.psb):
                        n = torch.randn(x.shape, generator=g, device="cuda", dtype=torch.float64)
                        x.mul_(1.0 + kick * n)
            runs[name] = snaps
            del m, stp
        rec = {"members": E, "dt_s": delt, "strictly_linear": lin, "heating_seed": seed,
               "kick": kick}
        for d in sorted(days):
            r = runs["fp64"][d]
            for name in ("fp64_input_rounded", "fp64_kicked_day10", "fp32", "bf16x3"):
                x = runs[name][d]
                if r is None or x is None:
                    rec[f"{name}_day{d}"] = "non-finite"
                    continue
                e, mem = {}, None
                for k in r:
                    e[k] = float(torch.linalg.norm(x[k] - r[k]) / torch.linalg.norm(r[k]))
                    dims = tuple(range(1, r[k].dim()))
                    pm = (torch.linalg.vector_norm(x[k] - r[k], dim=dims)
                          / torch.linalg.vector_norm(r[k], dim=dims))
                    mem = pm if mem is None else torch.maximum(mem, pm)
                e["members_within_1e-5"] = float((mem <= 1e-5).double().mean())
                e["member_median"] = float(mem.median())
                e["member_max"] = float(mem.max())
                e["worst_members"] = [int(i) for i in torch.argsort(mem, descending=True)[:5]]
                rec[f"{name}_day{d}"] = e
        out[label] = rec
        print(json.dumps({"conditioning_case": {label: rec}}), flush=True)
    return out


def adjoint_measurement(torch, days=20.0, snaps=None, fd_dirs=16, nsteps=None,
                        binomial_snaps=32, precision="fp64"):
    """Gradient of the area-mean day-20 streamfunction at sigma 0.25 over
    30-60N 150-210E with respect to the 20 x 64 x 128 heating (solid-body
    basic state, elliptic heating, plain damping, T42L20, FP64), by the
    checkpointed adjoint (every call's state stored when they fit in half
    the free device memory; also timed with ``binomial_snaps`` states on the
    binomial schedule); its time against the forward run of the same step
    (graph-replayed reference-layout calls) and against the fused FP64
    stepper's run, and central differences (eps 1e-4 relative) along seeded
    directions.  With ``precision="fp32"`` the adjoint, its forward run and
    the fused forward run are FP32, and the gradient is compared with the
    FP64 one instead of central differences (FP32 rounding swamps a
    1e-4 difference quotient)."""
    import types as _t
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid, configs
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    K = K_LEV
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heat = torch.as_tensor(configs.elliptic_heating(128, 64, sigm), device="cuda")
    sp, vg = Spectral(), VerticalGrid(sigm=sigm)
    mk = lambda nd, **kw: LBM(bs, sp, vg, Config(ndays=nd, **dict(configs.plain_damping(K),  # noqa
                                                                   **kw)))
    model = mk(days)
    resp64 = AreaMeanStreamfunction(sp, vg)

    def gradient(n=None, **kw):
        g = ForcingGradient(model, None, precision=precision, **(kw if n is None else
                                                                  dict(kw, nsteps=n)))
        g.response = resp64 if precision == "fp64" else AreaMeanStreamfunction(g.step.sp, vg)
        return g

    warm = gradient(4, snaps=2)
    warm.value_and_grad(heat)                        # captures every graph variant
    if nsteps is not None:
        days = nsteps / model.cfg.steps_per_day
    fg = gradient(ndays=days, snaps=snaps)
    fg._fg, fg._ag = warm._fg, warm._ag
    resp = fg.response

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    J_fwd, t_fwd = timed(lambda: fg.value(heat))
    (J, grad), t_grad = timed(lambda: fg.value_and_grad(heat))
    seq = gradient(ndays=days, snaps=snaps, pipeline=False)
    seq._fg, seq._ag = warm._fg, warm._ag
    (_, grad_seq), t_seq = timed(lambda: seq.value_and_grad(heat))
    del seq
    bino = gradient(ndays=days, snaps=binomial_snaps)
    bino._fg, bino._ag = warm._fg, warm._ag
    (_, grad_bino), t_bino = timed(lambda: bino.value_and_grad(heat))
    bino_steps = bino.forward_steps
    del bino
    sf = _t.SimpleNamespace(t=heat, vor=None, div=None, ps=None)
    m2 = mk(1.0, precision=precision)
    m2.run(steady_forcing=sf, verbose=False)          # warm-up (graph capture)
    m2.cfg.ndays = days
    _, t_fused = timed(lambda: m2.run(steady_forcing=sf, verbose=False))
    m3 = mk(days, precision=precision)
    m3.run(steady_forcing=sf, verbose=False)
    J_fused = float(resp64(m3.ga))
    vs64 = None
    if precision != "fp64":
        fd_dirs = 0
        g64 = ForcingGradient(model, resp64, ndays=days)
        J64, grad64 = g64.value_and_grad(heat)
        del g64
        vs64 = {"J_rel_diff": abs(float(J) - float(J64)) / abs(float(J64)),
                "grad_max_rel_diff": float((grad.double() - grad64).abs().max()
                                           / grad64.abs().max()),
                "grad_l2_rel_diff": float(torch.linalg.norm(grad.double() - grad64)
                                          / torch.linalg.norm(grad64))}
    rng = np.random.default_rng(16)
    hmax = float(heat.abs().max())
    fd = []
    for _ in range(fd_dirs):
        d = torch.as_tensor(rng.standard_normal(tuple(heat.shape)), device="cuda") * hmax
        e = 1e-4
        num = (float(fg.value(heat + e * d)) - float(fg.value(heat - e * d))) / (2 * e)
        adj = float((grad * d).sum())
        fd.append(abs(num - adj) / abs(num))
    calls = len(fg.calls)
    return {
        "workload": "T42L20 solid-body basic state, elliptic heating (0N 120E), plain damping, "
                    f"{precision.upper()}, 20 days (1440 steps + 2 start-up calls); response: "
                    "area-mean psi' at sigma 0.25, 30-60N x 150-210E, day 20",
        "precision": precision,
        "J": float(J), "J_forward_run": float(J_fwd), "J_fused_run": J_fused,
        "snaps": fg.snaps, "peak_stored_states": fg.peak_stored, "calls": calls,
        "stored_state_bytes": fg.state_bytes(),
        "forward_steps_in_gradient": fg.forward_steps,
        "forward_s": t_fwd, "gradient_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
        "gradient_one_stream_s": t_seq,
        "one_stream_vs_two_max_rel_diff": float((grad_seq - grad).abs().max()
                                                / grad.abs().max()),
        "fused_forward_s": t_fused, "gradient_over_fused_forward": t_grad / t_fused,
        "binomial": {"snaps": binomial_snaps, "forward_steps_in_gradient": bino_steps,
                     "gradient_s": t_bino, "gradient_over_forward": t_bino / t_fwd,
                     "gradient_over_fused_forward": t_bino / t_fused,
                     "max_rel_diff_vs_all_stored": float((grad_bino - grad).abs().max()
                                                         / grad.abs().max())},
        "fd_rel_err": fd, "fd_max_rel_err": max(fd) if fd else None,
        "vs_fp64_gradient": vs64,
        "grad_absmax": float(grad.abs().max()),
    }


def adjoint_batched_measurement(torch, nmem, nsteps, snaps=None, precision="fp64"):
    """One gradient of ``nmem`` members (seeded ensemble heatings, T42L20,
    each member its own response) reversed together, against one
    single-member gradient over the same calls, in `precision`."""
    from lbm_isca_gb300 import LBM, Config, Spectral, VerticalGrid, configs
    from lbm_isca_gb300.adjoint import AreaMeanStreamfunction, ForcingGradient
    from lbm_isca_gb300.ensemble import make_ensemble_model
    K = K_LEV
    sigm = configs.equal_sigma_half_levels(K)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    heats = torch.as_tensor(configs.ensemble_heating(128, 64, sigm, nmem, seed=SEED)[0],
                            device="cuda")
    cfg = lambda: Config(**configs.plain_damping(K))   # noqa: E731
    out = {"members": nmem, "calls": nsteps + 2}
    runs = (("single", None), ("batched", nmem))
    for name, E in runs:
        if E is None:
            sp, vg = Spectral(), VerticalGrid(sigm=sigm)
            m = LBM(bs, sp, vg, cfg())
            h = heats[0]
        else:
            m, sp, vg = make_ensemble_model(bs, E, cfg(), device="cuda", sigm=sigm)
            h = heats
        def make(n, **kw):
            g = ForcingGradient(m, None, nsteps=n, precision=precision, **kw)
            g.response = AreaMeanStreamfunction(g.step.sp, vg)
            return g
        warm = make(4, snaps=2)
        warm.value_and_grad(h)
        fg = make(nsteps, snaps=snaps)
        fg._fg, fg._ag = warm._fg, warm._ag
        out[f"{name}_snaps"] = fg.snaps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, g = fg.value_and_grad(h)
        torch.cuda.synchronize()
        out[f"{name}_gradient_s"] = time.perf_counter() - t0
        out[f"{name}_J0"] = float(J.reshape(-1)[0])
        out[f"{name}_grad0_absmax"] = float(g.reshape((-1,) + tuple(g.shape[-3:]))[0].abs().max())
    out["member_gradients_per_s_single"] = 1.0 / out["single_gradient_s"]
    out["member_gradients_per_s_batched"] = nmem / out["batched_gradient_s"]
    out["speedup_per_member"] = (out["member_gradients_per_s_batched"]
                                 / out["member_gradients_per_s_single"])
    return out


TC_OFF = -1


def main():
    global TC_OFF
    args = parse()
    TC_OFF = args.tc_off
    if args.adjoint and args.adjoint_members:
        import torch
        torch.cuda.set_device(0)
        out = adjoint_batched_measurement(torch, args.adjoint_members,
                                          args.adjoint_steps or 72,
                                          precision=args.adjoint_precision)
        print(json.dumps({"adjoint_batched": out}), flush=True)
        return
    if args.adjoint:
        import torch
        torch.cuda.set_device(0)
        out = adjoint_measurement(torch, fd_dirs=args.fd_dirs, nsteps=args.adjoint_steps,
                                  precision=args.adjoint_precision)
        print(json.dumps({"adjoint": out}), flush=True)
        return
    if args.uneven_groups:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"uneven_groups": uneven_groups_measurement(
            torch, args.precision, adjoint=args.adjoint_precision if args.uneven_groups_adjoint
            else None)}), flush=True)
        return
    if args.cpu_plans:
        print(json.dumps({"cpu_plans": cpu_plans()}), flush=True)
        return
    if args.conditioning:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps({"conditioning": conditioning(torch)}), flush=True)
        return
    if args.sweep:
        import torch
        torch.cuda.set_device(0)
        sw = precision_sweep(torch)
        worst = {}
        for r in sw.values():
            for key, e in r.items():
                if isinstance(e, dict) and "vor" in e:
                    prec = key.rsplit("_day", 1)[0]
                    worst[prec] = max(worst.get(prec, 0.0),
                                      max(e[k] for k in ("vor", "div", "t", "pi")))
        print(json.dumps({"precision_sweep": sw, "max_rel_l2": worst}), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return

    # CPU baseline first, before any CUDA call (spawned pool, rank 0, N = 1)
    cpu = None
    if rank == 0 and world == 1 and not args.no_extras:
        cores = min(host_cores(), 64)
        rate, res = cpu_oracle_throughput(cores, 1, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{cores} concurrent single-thread numpy oracle runs of one T42L20 "
                         f"member each, {min(n for n, _ in res)}+ steps in "
                         f"{args.cpu_seconds:.0f} s"}

    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from lbm_isca_gb300 import _lib
    from lbm_isca_gb300._lib import StepCtl, check, lib
    from lbm_isca_gb300.backend import stream_handle
    import ctypes as C

    E = args.members
    model, heats = build_model(E, args.precision, torch, seed=SEED + rank)
    from lbm_isca_gb300.ensemble import EnsembleForcing
    stp = model.stepper()
    delt = model.cfg.delt
    sched = model._schedule(args.warmup + args.steps + 1)
    stp.set_timesteps(sorted({dt for dt, _ in sched}))
    frc = model._spec_forcing(torch.as_tensor(heats, device="cuda"), True)
    stp.set_forcing(frc_t=frc, per_member=True)
    model._load_stepper(stp)
    # forward start + warm-up (the first advancing step carries ps_mode 1)
    n_start = model.cfg.inistp + 1
    stp.run(sched[:n_start], use_graph=False)
    stp.run(sched[n_start:n_start + args.warmup], use_graph=True)
    torch.cuda.synchronize()

    # ---- timed region: K steps, per-kernel CUDA events on the stepper stream ----
    planned, _ = stp.plan([(delt, False)] * args.steps)
    ctl = stp._ctl(planned[:1])
    d = stp.desc()
    L = lib()
    sh = stream_handle(stp.stream)
    # kernel ids of lbm_stepper_launch in step order
    fp32s = args.precision != "fp64"          # FP32 state (fp32 and the bf16 modes)
    kids = [4, 5, 6, 1, 2, 3] if fp32s else [0, 1, 2, 3]
    names = (["idft", "alg", "fdft"] if fp32s else ["grid"]) + \
        ["anal", "implicit", "synth"]
    nk = len(kids)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(nk + 1)]
           for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_wall = time.perf_counter()
        with torch.cuda.stream(stp.stream):
            for s in range(args.steps):
                ev = evs[s]
                ev[0].record(stp.stream)
                for i, kern in enumerate(kids):
                    check(L.lbm_stepper_launch(C.byref(d), ctl, kern, sh), "launch")
                    ev[i + 1].record(stp.stream)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    stp.pending_ps_mode = 2
    if world > 1:
        dist.barrier()
    total_ms = evs[0][0].elapsed_time(evs[-1][nk])
    kern_ms = np.zeros(nk)
    for ev in evs:
        for i in range(nk):
            kern_ms[i] += ev[i].elapsed_time(ev[i + 1])
    kern_ms /= args.steps
    t_max = total_ms
    if world > 1:
        tt = torch.tensor([total_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = world * E * args.steps / (t_max / 1000.0)
    finite = stp.check_finite()

    # ---- graph replay of the same steps (informational) ----
    torch.cuda.synchronize()
    g0 = torch.cuda.Event(enable_timing=True)
    g1 = torch.cuda.Event(enable_timing=True)
    g0.record(stp.stream)
    stp.run([(delt, False)] * args.steps, use_graph=True, graph_chunk=72)
    g1.record(stp.stream)
    torch.cuda.synchronize()
    graph_ms = g0.elapsed_time(g1) / args.steps

    # ---- end to end through the public API, host buffers ----
    e2e = None
    if rank == 0:
        e2e = end_to_end(args, E, heats, torch)

    # ---- extras: accuracy vs FP64 and the plain single-member FP64 rate ----
    # (N = 1 only, like the CPU baseline: the FP64 reference over all members
    # and 30 days takes minutes, which other ranks must not wait through)
    extras = {}
    if rank == 0 and world == 1 and not args.no_extras:
        extras = side_measurements(args, torch)

    if rank == 0:
        p = 4 if fp32s else 8
        ab = algorithmic_bytes(E, p)
        top = int(np.argmax(kern_ms))
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except Exception:
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        achieved = ab[names[top]] / (kern_ms[top] / 1000.0) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPES[args.precision], "data": "synthetic",
            "config": {"workload": f"{E}-member T42L20 ensemble (solid-body basic state, "
                                   f"seeded elliptic heatings seed {SEED}+rank, plain "
                                   f"damping), FP32 state, fused stepper; {placement(stp)}",
                       "members_per_gpu": E, "grid": "T42 128x64 Gaussian",
                       "levels": "L20 equal sigma", "dt_s": delt,
                       "l2": "inputs larger than L2 (per-step working set "
                             f"{sum(ab.values()) / 1e9:.2f} GB)",
                       "parallelism": f"members sharded, {world} independent rank(s)"},
            "clocks": clk.summary(),
            "e2e": e2e,
            "gpu_launches": stp.launches_per_step() * args.steps,
            "roofline": {"bound": "hbm", "kernel": names[top], "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": read_traffic(traffic_key(stp, names[top]), E),
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
            "roofline_step": step_roofline(E, p, t_max / args.steps, peaks, args.precision),
            "kernel_ms": dict(zip(names, [float(x) for x in kern_ms])),
            "kernel_share": dict(zip(names, [float(x / kern_ms.sum()) for x in kern_ms])),
            "algorithmic_gbs": {n: ab[n] / (kern_ms[i] / 1000.0) / 1e9
                                for i, n in enumerate(names)},
            "graph_ms_per_step": graph_ms,
            "wall_s_timed": t_wall,
            "finite": finite,
            "cpu_baseline": cpu,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def end_to_end(args, E, heats, torch):
    """The bench's steps through the public API with host buffers: the
    pinned host heatings are copied to the device, LBM.run integrates the
    ensemble (forcing analysis, state load, the steps, synthesis of the final
    grid state) and the final grid state is copied into pinned host buffers
    allocated beforehand, as a caller that reads every run's result keeps
    them.  One untimed run first (kernel loading, allocator growth); the
    timed run starts from the zero state again; a third run with
    Config.phase_timing (device synchronised at phase boundaries) gives the
    split by phase, reported beside the timed number."""
    from lbm_isca_gb300.ensemble import EnsembleForcing
    fields = ("u", "v", "t", "q", "ps")
    days = args.steps / 72.0
    m2, _ = build_model(E, args.precision, torch, days=days, seed=SEED)
    host_heat = torch.from_numpy(heats.astype(np.float64)).pin_memory()
    host_out = {k: torch.empty(tuple(getattr(m2.ga, k).shape), dtype=torch.float64,
                               pin_memory=True) for k in fields}

    def one_run(profile):
        for st in (m2.ga, m2.gb):
            for k in fields:
                getattr(st, k).zero_()
        m2.cfg.phase_timing = profile
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # H2D and D2H over the CPU-GPU link (SM loads / stores of pinned memory)
        dev_heat = torch.empty(tuple(host_heat.shape), device="cuda", dtype=host_heat.dtype)
        torch.ops.lbm_gb300.link_copy_(dev_heat, host_heat)
        m2.run(mjo_forcing=EnsembleForcing(dev_heat, device="cuda"), verbose=False)
        t1 = time.perf_counter()
        for k in fields:
            torch.ops.lbm_gb300.link_copy_(host_out[k], getattr(m2.ga, k).contiguous())
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return t2 - t0, t2 - t1

    one_run(False)
    t_e2e, _ = one_run(False)
    _, t_d2h = one_run(True)
    phases = dict(m2.phases or {})
    phases["d2h"] = t_d2h
    nb_in = host_heat.numel() * host_heat.element_size()
    nb_out = sum(x.numel() * x.element_size() for x in host_out.values())
    del m2
    return {"value": E * args.steps / t_e2e, "unit": UNIT,
            "h2d_bytes_per_step": nb_in / args.steps,
            "d2h_bytes_per_step": nb_out / args.steps,
            "seconds": t_e2e,
            "phases_s": phases,
            "note": "LBM.run of the ensemble from pinned host heatings (H2D inside), "
                    f"{args.steps} advancing + 2 start-up steps, final grid state copied "
                    "to pinned host buffers (D2H inside); both copies by lbm_link_copy "
                    "(SM loads/stores over NVLink-C2C); after one untimed run; "
                    "phases_s from a further run synchronised at phase boundaries"}


def accuracy_block(args, torch, E, days=(10, 30)):
    """Relative L2 per prognostic field of the bench's precision against FP64
    over every member of the timed ensemble (its heatings, seed 1) after 10
    and 30 days: one run of each precision through the fused stepper, the
    state taken at the end of day 10 (call 722) and of day 30 (call 2162);
    packed spectral coefficients of all members (vor, div, T: every level;
    pi), q' as its absolute maximum (it stays 0: no moisture forcing).  The
    FP32 FMA path on the same members is reported beside it, and per member
    (each member's relative L2, worst field) the share within 1e-5."""
    res = {}
    precs = ["fp64", args.precision] + (["fp32"] if args.precision != "fp32" else [])
    for prec in precs:
        t0 = time.perf_counter()
        m, heats = build_model(E, prec, torch, days=max(days))
        stp = m.stepper()
        sched = m._schedule(72 * max(days))
        stp.set_timesteps(sorted({dt for dt, _ in sched}))
        stp.set_forcing(frc_t=m._spec_forcing(torch.as_tensor(heats, device="cuda"), True),
                        per_member=True)
        stp.load_zero()
        snaps, done = {}, 0
        for d in sorted(days):
            upto = 72 * d + m.cfg.inistp
            stp.run(sched[done:upto], use_graph=True)
            done = upto
            torch.cuda.synchronize()
            # copies: .to() of an FP64 state would return a view of it
            snaps[d] = {k: x.to(torch.complex128, copy=True) for k, x in
                        (("vor", stp.sa3[:, 0]), ("div", stp.sa3[:, 1]), ("t", stp.sa3[:, 2]),
                         ("pi", stp.sas[:, 0]), ("q", stp.sa3[:, 3]))}
        if not stp.check_finite():
            raise FloatingPointError(f"accuracy run in {prec} produced non-finite values")
        res[prec] = snaps
        del m, stp
        print(f"accuracy run {prec}: {time.perf_counter() - t0:.1f} s", file=sys.stderr,
              flush=True)
    out, worst = {}, {}
    for prec in precs[1:]:
        tag = "" if prec == args.precision else f"_{prec}"
        for d in sorted(days):
            rel, mem = {}, None
            for k in ("vor", "div", "t", "pi"):
                r, f = res["fp64"][d][k], res[prec][d][k]
                rel[k] = float(torch.linalg.norm(f - r) / torch.linalg.norm(r))
                dims = tuple(range(1, r.dim()))
                pm = torch.linalg.vector_norm(f - r, dim=dims) / torch.linalg.vector_norm(r, dim=dims)
                mem = pm if mem is None else torch.maximum(mem, pm)
                if prec == args.precision:
                    worst[d] = max(worst.get(d, 0.0), rel[k])
            rel["q_absmax"] = float(res[prec][d]["q"].abs().max())
            rel["members_within_1e-5"] = float((mem <= 1e-5).double().mean())
            rel["member_median"] = float(mem.median())
            rel["member_max"] = float(mem.max())
            out[f"accuracy{tag}_vs_fp64_day{d}"] = rel
    out["accuracy_max_rel_l2"] = {f"day{d}": v for d, v in worst.items()}
    out["accuracy_within_1e-5"] = {f"day{d}": bool(v <= 1e-5) for d, v in worst.items()}
    out["accuracy_members"] = E
    return out


def side_measurements(args, torch):
    """FP32-vs-FP64 relative L2 per prognostic field after 10 and 30 days over
    every member of the timed ensemble, and the plain single-member FP64 GPU
    rate that the batched rate is compared with."""
    out = accuracy_block(args, torch, args.members)
    # plain single-member FP64 GPU path
    m1, heats = build_model(1, "fp64", torch, days=1.0)
    stp = m1.stepper()
    sched = m1._schedule(200)
    stp.set_timesteps(sorted({dt for dt, _ in sched}))
    stp.set_forcing(frc_t=m1._spec_forcing(torch.as_tensor(heats, device="cuda"), True),
                    per_member=True)
    m1._load_stepper(stp)
    stp.run(sched[:3], use_graph=False)
    stp.run([(m1.cfg.delt, False)] * 20, use_graph=True)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    n = 200
    e0.record(stp.stream)
    stp.run([(m1.cfg.delt, False)] * n, use_graph=True)
    e1.record(stp.stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    out["plain_fp64_single_member"] = {"ms_per_step": ms, "member_steps_per_s": 1000.0 / ms}
    return out


if __name__ == "__main__":
    main()

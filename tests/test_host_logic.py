"""Host-side logic that needs no GPU: step schedule, ps-filter bookkeeping,
synthetic inputs, device selection, member sharding (2 gloo ranks)."""

import os
import socket
import types

import numpy as np
import pytest

from lbm_isca_gb300 import configs
from lbm_isca_gb300.sharding import member_block


def test_schedule_matches_reference_loop():
    """model.py:213-219: inistp start-up calls at dt/2^(inistp-istep+1)."""
    from lbm_isca_gb300.model import LBM, Config
    fake = types.SimpleNamespace(cfg=Config(delt=1200.0, inistp=2))
    sched = LBM._schedule(fake, 5)
    assert sched[:2] == [(300.0, True), (600.0, True)]
    assert sched[2:] == [(1200.0, False)] * 5
    fake.cfg.inistp = 0
    assert LBM._schedule(fake, 3) == [(1200.0, False)] * 3


def test_ps_mode_plan():
    """Grid-ps filter bookkeeping: first step 0, after a start-up call 1
    (copy), after an advancing call 2 (Robert-Asselin)."""
    from lbm_isca_gb300.stepper import EnsembleStepper
    fake = types.SimpleNamespace(pending_ps_mode=0)
    steps = [(300.0, True), (600.0, True), (1200.0, False), (1200.0, False)]
    planned, pend = EnsembleStepper.plan(fake, steps)
    assert [p[2] for p in planned] == [0, 1, 1, 2]
    assert pend == 2
    fake.pending_ps_mode = 2
    planned, pend = EnsembleStepper.plan(fake, [(1200.0, False)])
    assert planned == [(1200.0, False, 2)] and pend == 2


def test_heating_profile_peaks_at_sigma_peak():
    sig = np.linspace(0.0, 1.0, 100001)
    for sp in (0.3, 0.45, 0.6):
        prof = configs.heating_profile(sig, sp)
        assert abs(sig[np.argmax(prof)] - sp) < 1e-4
        assert abs(prof[0]) < 1e-12 and abs(prof[-1]) < 1e-12


def test_elliptic_heating_and_ensemble_draws():
    sigm = configs.equal_sigma_half_levels(20)
    h = configs.elliptic_heating(128, 64, sigm)
    assert h.shape == (64, 128, 20)
    assert 0.0 < h.max() <= 2.0 / 86400.0 + 1e-18
    _, lat = configs.gaussian_latitudes(64)
    lon = np.arange(128) * 360.0 / 128
    j, i, _ = np.unravel_index(np.argmax(h), h.shape)
    assert abs(lat[j]) < 3.0 and abs(lon[i] - 120.0) <= 2.9
    assert h[np.abs(lat) > 10.0].max() == 0.0           # compact support
    e1, p1 = configs.ensemble_heating(64, 32, sigm, 3, seed=7)
    e2, p2 = configs.ensemble_heating(64, 32, sigm, 3, seed=7)
    assert np.array_equal(e1, e2) and p1 == p2
    for lon0, lat0, amp, sp in p1:
        assert 0 <= lon0 < 360 and -15 <= lat0 <= 15 and amp > 0 and 0.3 <= sp <= 0.6


def test_solid_body_state_is_balanced_and_monotone():
    sigm = configs.equal_sigma_half_levels(20)
    bs = configs.solid_body_basic_state(128, 64, sigm)
    mu, _ = configs.gaussian_latitudes(64)
    assert np.allclose(bs.u[:, 0, 0], 15.0 * np.sqrt(1 - mu ** 2))
    assert bs.v.max() == 0.0 and bs.q.max() == 0.0
    t = bs.t[0, 0]
    assert np.all(np.diff(t) <= 0.0) and t.min() >= configs.T_FLOOR
    assert bs.ps.max() <= configs.PS_EQUATOR_HPA + 1e-9


def test_plain_damping_profile():
    kw = configs.plain_damping(20)
    assert kw["ddragv"][0] == 1.0 and kw["ddragv"][-1] == 1.0
    assert kw["ddragv"][1:-1] == [30.0] * 18
    assert kw["sponge"] is False and kw["vdifv"] is None and kw["hdif_tefold"] == 6.0


def test_backend_without_a_gpu():
    torch = pytest.importorskip("torch")
    from lbm_isca_gb300.backend import resolve
    with pytest.raises(ValueError):
        resolve("tpu")
    with pytest.raises(RuntimeError):
        resolve("cpu")
    if not torch.cuda.is_available():
        with pytest.raises(RuntimeError):
            resolve("gb300")


def test_member_block_partition():
    for total in (1, 7, 96, 512):
        for world in (1, 2, 3, 8):
            blocks = [member_block(total, world, r) for r in range(world)]
            assert sum(c for _, c in blocks) == total
            pos = 0
            for first, count in blocks:
                assert first == pos
                pos += count


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, total, out_dir):
    """Each rank integrates its member block with the oracle (T21, 6 steps)
    and the blocks are gathered over gloo."""
    import torch
    import torch.distributed as dist
    from oracle import lbm_oracle as orc
    from lbm_isca_gb300.sharding import gather_members
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = member_block(total, world, rank)
    sigm = configs.equal_sigma_half_levels(20)
    heats, _ = configs.ensemble_heating(64, 32, sigm, total, seed=3)
    tr = orc.SphericalTransform(64, 32, 21)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(20)), nmem=count)
    m.run(4, frc_t=heats[first:first + count])
    local = torch.as_tensor(m.ga.t)
    full = gather_members(local, world)
    if rank == 0:
        np.save(os.path.join(out_dir, "full.npy"), full.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_members_match_single_process(tmp_path):
    """2 gloo ranks, 3 members split 2 + 1: identical to one 3-member run."""
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    port = _free_port()
    tmp.spawn(_rank_main, args=(2, port, 3, str(tmp_path)), nprocs=2, join=True)
    full = np.load(os.path.join(tmp_path, "full.npy"))
    from oracle import lbm_oracle as orc
    sigm = configs.equal_sigma_half_levels(20)
    heats, _ = configs.ensemble_heating(64, 32, sigm, 3, seed=3)
    tr = orc.SphericalTransform(64, 32, 21)
    lv = orc.SigmaLevels(sigm)
    bs = configs.solid_body_basic_state(64, 32, sigm)
    m = orc.OracleModel(tr, lv, bs, orc.RunConfig(**configs.plain_damping(20)), nmem=3)
    m.run(4, frc_t=heats)
    assert full.shape == m.ga.t.shape
    assert np.abs(full - m.ga.t).max() <= 1e-12 * np.abs(m.ga.t).max()


def test_mjo_forcing_call_sequence_and_plan():
    """MJOForcing follows forcing.py:99-157 (spin-up hold, then linear
    interpolation over nt calls per day); plan() names the field the next
    step() returns."""
    import numpy as np
    from lbm_isca_gb300.forcing import MJOForcing
    gtf = np.arange(3)[:, None, None, None] * np.ones((3, 2, 4, 5)) + 1.0
    f = MJOForcing(gtf, nt=4, spinup=3)
    for call in range(1, 20):
        a, b, w = f.plan()
        got = f.step()
        want = gtf[a] + (gtf[b] - gtf[a]) * w
        assert np.allclose(got, want), call
    # spin-up holds day 1, then day 1 -> day 2 over 4 calls, ...
    f.reset()
    vals = [float(f.step()[0, 0, 0]) for _ in range(12)]
    assert vals[:2] == [1.0, 1.0]
    assert vals[2:6] == [1.0, 1.25, 1.5, 1.75]
    assert vals[6:10] == [2.0, 2.25, 2.5, 2.75]
    assert vals[10:12] == [3.0, 3.0]


def test_tensor_core_table_image_layout():
    """The tc_anal table image: every element sits at the byte the header
    gives, (m, s) blocks in order, three tables x three bfloat16 pieces per
    block, and the pieces sum to the FP64 table to 2^-24 (checked on the CPU
    against the oracle's tables)."""
    import torch
    from oracle import lbm_oracle as orc
    from lbm_isca_gb300.stepper import tc_anal_image
    N, J = 21, 32
    tr = orc.SphericalTransform(64, 32, N)
    P, H = torch.as_tensor(tr.P), torch.as_tensor(tr.H)
    nn1a = torch.as_tensor(-tr.lap)
    img = tc_anal_image(P, H, nn1a, N).numpy().view(np.uint16)
    tabs = (tr.P, tr.H, tr.P * (-tr.lap)[None, :, None])
    KS = J // 16

    def bf16(u):      # bfloat16 bits -> float
        return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
    base = 0
    rng = np.random.default_rng(0)
    for m in range(N + 1):
        nr = N + 1 - m
        nb = (nr + 15) // 16 * 16
        for _ in range(40):
            s, t = rng.integers(KS), rng.integers(3)
            r, kk = rng.integers(nb), rng.integers(16)
            tile = base + s * 9 * nb * 16
            off = (r // 8) * 128 + (kk // 8) * 64 + (r % 8) * 8 + kk % 8
            val = sum(bf16(img[tile + (t * 3 + p) * nb * 16 + off]) for p in range(3))
            ref = tabs[t][m, m + r, s * 16 + kk] if r < nr else 0.0
            assert abs(val - ref) <= 2.0 ** -24 * abs(ref) + 1e-36, (m, s, t, r, kk)
        base += KS * 9 * nb * 16
    assert base == img.size


def test_tensor_core_synthesis_table_image_layout():
    """The tc_synth table image: (m, part, step) blocks in order, the tables
    m P il, -H il, H il, P as latitude x 16-row tiles, pieces summing to the
    FP64 values (checked on the CPU against the oracle's tables)."""
    import torch
    from oracle import lbm_oracle as orc
    from lbm_isca_gb300.stepper import tc_synth_image
    for (nlon, nlat, N) in ((64, 32, 21), (256, 128, 85)):
        tr = orc.SphericalTransform(nlon, nlat, N)
        J = nlat
        nparts = 1 if 6 * J <= 512 else 2
        JT = J // nparts
        il = tr.invlap
        img = tc_synth_image(torch.as_tensor(tr.P), torch.as_tensor(tr.H),
                             torch.as_tensor(il), N).numpy().view(np.uint16)

        def bf16(u):
            return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        rng = np.random.default_rng(1)
        base = 0
        for m in range(N + 1):
            nr = N + 1 - m
            ks = (nr + 15) // 16
            tabs = (m * tr.P[m] * il[:, None], -tr.H[m] * il[:, None], tr.H[m] * il[:, None],
                    tr.P[m])
            for part in range(nparts):
                for _ in range(12):
                    s, t = rng.integers(ks), rng.integers(4)
                    r, kk = rng.integers(JT), rng.integers(16)
                    n = m + 16 * s + kk
                    blk = base + (part * ks + s) * 12 * JT * 16
                    off = (r // 8) * 128 + (kk // 8) * 64 + (r % 8) * 8 + kk % 8
                    val = sum(bf16(img[blk + (t * 3 + p) * JT * 16 + off]) for p in range(3))
                    ref = tabs[t][n, part * JT + r] if n <= N else 0.0
                    assert abs(val - ref) <= 2.0 ** -24 * abs(ref) + 1e-36, (m, part, s, t, r)
            base += nparts * ks * 12 * JT * 16
        assert base == img.size


def test_tensor_core_longitude_table_image_layout():
    """The tc_dft table image: per 16-longitude step three bfloat16 pieces of
    the 128 x 16 tile W[2m][i] = cos(2 pi m i / I) / I, W[2m+1][i] =
    -sin(2 pi m i / I) / I (zero past nmax), each element at the byte the
    header gives, pieces summing to the FP64 value to 2^-24; then the FP32
    cos(2 pi t / I) table of the surface rows."""
    from lbm_isca_gb300.stepper import tc_dft_image
    for (I, N) in ((64, 21), (128, 42)):
        img = tc_dft_image(N, I).numpy().view(np.uint16)
        KS = I // 16
        assert img.size == KS * 3 * 128 * 16 + 2 * I
        cs = img[KS * 3 * 128 * 16:].copy().view(np.float32)
        assert np.array_equal(cs, np.cos(2.0 * np.pi * np.arange(I) / I).astype(np.float32))

        def bf16(u):
            return (u.astype(np.uint32) << 16).view(np.float32).astype(np.float64)
        for s in range(KS):
            for L in range(128):
                for kk in range(16):
                    m, c, i = L // 2, L % 2, 16 * s + kk
                    ang = 2.0 * np.pi * ((m * i) % I) / I
                    ref = 0.0 if m > N else (np.cos(ang) if c == 0 else -np.sin(ang)) / I
                    off = (L // 8) * 128 + (kk // 8) * 64 + (L % 8) * 8 + kk % 8
                    val = sum(bf16(img[(s * 3 + p) * 2048 + off]) for p in range(3))
                    assert abs(val - ref) <= 2.0 ** -24 * abs(ref) + 1e-36, (I, s, L, kk)


def test_autotune_candidates_keep_the_precision_placement():
    """bf16x3 never clears the Legendre bits (their tensor-core accumulation
    breaks its 1e-5 gate); bf16split may place every contraction; the
    longitude-analysis bit is free only where its tensor-core table exists."""
    import types
    from lbm_isca_gb300.autotune import candidates
    mk = lambda prec, dft: types.SimpleNamespace(K=20, E=32, precision=prec,   # noqa: E731
                                                 tc_dft=object() if dft else None)
    c3 = candidates(mk("bf16x3", True))
    assert c3 and all(off & 3 == 3 for off, _ in c3)
    assert {off for off, _ in c3} == {3, 7}
    cs = candidates(mk("bf16split", True))
    assert {off for off, _ in cs} == set(range(8))
    assert {g for _, g in cs} == {0, 3, 1}
    assert all(off & 4 for off, _ in candidates(mk("bf16split", False)))


def test_launches_per_step():
    """FP64: four kernels; FP32: six; each contraction on the tensor cores
    adds the launch of its surface fields' FMA kernel."""
    import types
    from lbm_isca_gb300.stepper import EnsembleStepper
    f = EnsembleStepper.launches_per_step
    ns = lambda prec, leg, off, dft: types.SimpleNamespace(   # noqa: E731
        precision=prec, legendre=leg, tc_off=off, tc_dft=object() if dft else None)
    assert f(ns("fp64", 0, 0, False)) == 4
    assert f(ns("fp32", 0, 0, False)) == 6
    assert f(ns("bf16x3", 6, 3, True)) == 7
    assert f(ns("bf16x3", 6, 0, True)) == 9
    assert f(ns("bf16split", 3, 0, False)) == 8
    assert f(ns("bf16x3", 6, 7, True)) == 6

"""GPU: the reference's configurations themselves, through the C ABI, against the oracle.

* Batched configuration (L = 32, 64 disorder configurations x 32-replica ladders over
  T = 8.0-11.5, PHI = 2, XI = 3): the production FP32 kernel (the shape-specialised,
  shared-memory-resident sweep kernel with packed FP32x2 arithmetic) is the one the autotuner
  keeps; its flip decisions against the oracle's FP64 replay of the same sweeps from the same
  state; its thermal averages against the FP64 form's on the same seeds.
* Plain LOCAL configuration (L = 16, T = 9.5, one lattice, 10^4 + 10^4 sweeps) and plain PT
  configuration (L = 24, 16 replicas, stripe start along x): the FP64 form bit-identical to the
  oracle's replay over the whole run.

The acceptance rule that the FP32 decision is checked against is Metro_sweep's
(sim/J1J2_6tv.f90:2572-2604): accept if dE <= 0, else if u < exp(-beta dE).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 1
L3, NCONF3, NREP3 = 32, 64, 32
OBS = ("absmag", "mag2", "en", "en2", "strx_abs", "stry_abs", "nbar", "nbar2")


def _betas(nrep, tmin=8.0, tmax=11.5):
    from oracle import oracle as O
    return 1.0 / O.ladder(nrep, tmin, tmax)


def _batched_engine(jc, precision):
    eng = jc.Engine(L3, L3, nconf=NCONF3, nreplica=NREP3, ptswapever=5, precision=precision,
                    seed=SEED)
    betas = _betas(NREP3)
    for k in range(NCONF3):
        eng.set_disorder(k, jc.disorder(L3, L3, SEED + k))
        eng.set_ladder(k, betas)
        eng.init_spins(k, jc.START_HOT)
    eng.reset_measurements()
    return eng, betas


def test_batched_fp32_kernel_decisions_match_fp64_replay(engine_mod, oracle):
    """One PT cycle (PTSWAPEVER = 5 sweeps) of the production FP32 kernel from an equilibrated
    state, against the oracle's FP64 replay of the same five sweeps (same colour order, Philox
    words and temperatures) from the same state: per-site disagreements below 1e-4 of the sites
    (a mismatched decision also changes its neighbours' later fields, so this bounds the
    decision mismatch rate from above)."""
    jc = engine_mod
    eng, betas = _batched_engine(jc, jc.FP32_BATCHED)
    eng.run(50, measure=False)  # equilibrate (the tuner has picked the kernel by now)
    cfg = eng.config()
    # the shape-specialised kernel: one or two lattices (32 KiB each) and their FP32 field
    # (128 KiB) in shared memory, a spin word (four sites) per thread and colour phase
    assert cfg["smem_bytes"] in (L3 ** 3 + 4 * L3 ** 3, 2 * L3 ** 3 + 4 * L3 ** 3), cfg
    assert cfg["sites_per_thread"] == 4 and cfg["block_threads"] in (512, 1024), cfg
    confs = (0, 21, 42, 63)
    before = {(k, r): eng.spins(k, r).copy() for k in confs for r in range(NREP3)}
    tors = {k: eng.maps(k)[1] for k in confs}
    eng.run(1, measure=False)
    sweep0 = 50 * 5
    diff = flips = sites = 0
    for k in confs:
        M = oracle.Model(L3, L3, jc.disorder(L3, L3, SEED + k))
        for r in range(NREP3):
            s = before[(k, r)].copy()
            flips += M.replay_sweeps(s, betas[tors[k][r]], SEED, k, r, sweep0, 5)
            got = eng.spins(k, r)
            diff += int((got != s).sum())
            sites += s.size
    rate = diff / sites
    print(f"FP32 kernel vs FP64 replay, one PT cycle of {len(confs) * NREP3} lattices: "
          f"{diff} of {sites} sites differ ({rate:.2e}); {flips} accepted flips in the replay")
    assert flips > 0
    assert rate <= 1e-4
    eng.close()


def test_batched_fp32_observables_within_two_sigma_of_fp64(engine_mod, oracle):
    """The batched configuration in both forms from the same starts and streams, 300 + 2000 PT
    cycles; for each temperature slot and each of |m|, m^2, E, E^2, |strx|, |stry|, nbar, nbar^2
    (256 comparisons):

    * error bars: |FP32 - FP64| of the disorder averages against the error bar the reference's
      output files carry for such an average (std over configurations / sqrt(NCONF),
      J:3210-3575) of each form, combined.  Every |z| < 3 and at most 2 % above 2.  (Where the
      spread over configurations is mostly thermal, as for |m| and m^2 here, an unbiased FP32
      form still puts about 1 in 200 of these z beyond 2, so "every |z| < 2" over 256
      comparisons would fail one clean run in three.)
    * paired: the same difference against its own standard error over the 64 configurations
      (the disorder spread cancels), a much sharper test for a bias: t distributed with 63
      degrees of freedom if both forms sample the same distribution, neighbouring slots
      correlated through the replica exchange; none above 4.5 (chance 256 * 2.9e-5), at most
      15 % above 2 (5 % expected)."""
    jc = engine_mod
    cols = [jc.SUM_FIELDS.index(n) for n in OBS]
    nmess = 2000
    avg = {}
    for prec in (jc.FP64_PLAIN, jc.FP32_BATCHED):
        eng, _ = _batched_engine(jc, prec)
        eng.run(300, measure=False)
        eng.reset_measurements()
        eng.run(nmess, measure=True)
        s, nm = eng.slot_sums(-1)
        assert (nm == nmess).all()
        avg[prec] = (s[:, cols] / nm[:, None]).reshape(NCONF3, NREP3, len(OBS))
        eng.close()
    a32, a64 = avg[jc.FP32_BATCHED], avg[jc.FP64_PLAIN]
    n = NCONF3
    delta = a32.mean(axis=0) - a64.mean(axis=0)
    err = np.sqrt(a32.var(axis=0, ddof=1) / n + a64.var(axis=0, ddof=1) / n)
    z = np.abs(delta) / err
    d = a32 - a64
    zp = np.abs(d.mean(axis=0)) / (d.std(axis=0, ddof=1) / np.sqrt(n))
    for j, name in enumerate(OBS):
        print(f"{name:9s} |z| (error bars) by slot:", " ".join(f"{v:.2f}" for v in z[:, j]))
        print(f"{name:9s} |z| (paired)     by slot:", " ".join(f"{v:.2f}" for v in zp[:, j]))
    print(f"error bars: max |z| {z.max():.3f}, {(z > 2).sum()} of {z.size} above 2; "
          f"paired: max {zp.max():.3f}, {(zp > 2).sum()} of {zp.size} above 2")
    assert z.max() < 3, z
    assert (z > 2).mean() <= 0.02, z
    assert zp.max() < 4.5, zp
    assert (zp > 2).mean() <= 0.15, zp


def test_local_configuration_fp64_bit_identical_over_1e4_sweeps(engine_mod, oracle):
    """LOCAL sampler, L = 16, T = 9.5, PHI = 2, XI = 3, seed 1, HOT start: 10^4 equilibration
    and 10^4 measured sweeps (one sweep per cycle, no swaps) bit-identical to the oracle's
    replay: spins, running sums, observables; the final m, strx, stry equal the reference's own
    Measurement of the configuration."""
    jc = engine_mod
    L, beta = 16, 1.0 / 9.5
    p = jc.disorder(L, L, SEED)
    eng = jc.Engine(L, L, nconf=1, nreplica=1, ptswapever=1, precision=jc.FP64_PLAIN, seed=SEED)
    eng.set_disorder(0, p)
    eng.set_ladder(0, np.array([beta]))
    eng.init_spins(0, jc.START_HOT)
    eng.reset_measurements()
    st = oracle.new_pt_state(eng.spins(0, 0)[None, :].copy())
    eng.run(10000, measure=False, restart_swap_phase=True)
    eng.reset_measurements()
    eng.run(10000, measure=True, restart_swap_phase=True)
    M = oracle.Model(L, L, p)
    M.replay_pt(st, [beta], 1, 10000, 0, SEED, 0, False, 1)
    obs = M.replay_pt(st, [beta], 1, 10000, 10000, SEED, 0, True, 1)
    s = eng.spins(0, 0)
    np.testing.assert_array_equal(s, st["spins"][0])
    sums, nm = eng.slot_sums(0)
    assert nm[0] == 10000
    np.testing.assert_array_equal(sums, st["sums"])
    np.testing.assert_array_equal(eng.observables(0), obs)
    ref = M.measurement(s)
    got = eng.observables(0)[0]
    assert got[0] == ref[0] and got[2] == ref[2] and got[3] == ref[3]
    assert abs(got[1] - ref[1]) < 1e-9
    eng.close()


def test_pt_configuration_stripe_start_fp64_bit_identical(engine_mod, oracle):
    """Plain PT configuration: L = 24, 16 replicas linear over T = 8.0-11.5, PHI = 2, XI = 3,
    START = STR with STRAXIS = X (the reference's Initialize_spin_array, J:1179-1209), 50
    equilibration + 200 measured PT cycles of 5 sweeps: slot maps, swap counters, visit flags,
    spins, running sums and observables bit-identical to the oracle's replay."""
    jc = engine_mod
    L, nrep = 24, 16
    betas = _betas(nrep)
    p = jc.disorder(L, L, SEED)
    eng = jc.Engine(L, L, nconf=1, nreplica=nrep, ptswapever=5, precision=jc.FP64_PLAIN,
                    seed=SEED)
    eng.set_disorder(0, p)
    eng.set_ladder(0, betas)
    eng.init_spins(0, jc.START_STR, jc.AXIS_X)
    eng.reset_measurements()
    stripes = oracle.init_spins(SEED, L, L, 2, 0)
    spins0 = np.stack([eng.spins(0, r) for r in range(nrep)])
    for r in range(nrep):
        np.testing.assert_array_equal(spins0[r], stripes)
    st = oracle.new_pt_state(spins0)
    neq, nmess = 50, 200
    eng.run(neq, measure=False, restart_swap_phase=True)
    eng.reset_measurements()
    eng.run(nmess, measure=True, restart_swap_phase=True)
    M = oracle.Model(L, L, p)
    M.replay_pt(st, betas, 5, neq, 0, SEED, 0, False, 1)
    obs = M.replay_pt(st, betas, 5, nmess, neq, SEED, 0, True, 1)
    rat, tor = eng.maps(0)
    np.testing.assert_array_equal(rat, st["rep_at_temp"])
    np.testing.assert_array_equal(tor, st["temp_of_rep"])
    for r in range(nrep):
        np.testing.assert_array_equal(eng.spins(0, r), st["spins"][r])
    sums, nm = eng.slot_sums(0)
    np.testing.assert_array_equal(nm, st["nmeas"])
    np.testing.assert_array_equal(sums, st["sums"])
    att, acc, vb = eng.pt_stats(0)
    np.testing.assert_array_equal(att, st["attempts"][:nrep - 1])
    np.testing.assert_array_equal(acc, st["accepts"][:nrep - 1])
    assert acc.sum() > 0
    assert vb == int(np.sum(st["visited"] == 3))
    np.testing.assert_array_equal(eng.observables(0), obs)
    eng.close()

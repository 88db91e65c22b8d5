"""GPU parity: the CUDA engine (through the C ABI) against the oracle.

* FP64 form: spins, observables, slot maps, swap counters and running sums bit-identical to the
  oracle's replay of the same colour order, Philox stream, exponential and fixed-point energy.
* FP32 form: per-site path == quad path bit for bit; decision mismatch rate against FP64 in
  deterministic replay; observables within statistical error of the FP64 form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 1


def _betas(nrep, tmin=8.0, tmax=11.5):
    from oracle import oracle as O
    return 1.0 / O.ladder(nrep, tmin, tmax)


def _setup(jc, O, L, H, nconf, nrep, precision, pp=0.0, bonds=0.0, flags=0, start=0, axis=0,
           seed=SEED, conf_base=0, ptswapever=5, betas=None, block_threads=0):
    eng = jc.Engine(L, H, nconf=nconf, nreplica=nrep, ptswapever=ptswapever, precision=precision,
                    seed=seed, conf_base=conf_base, flags=flags, block_threads=block_threads)
    betas = _betas(nrep) if betas is None else betas
    models = []
    for k in range(nconf):
        p = jc.disorder(L, H, seed + k)
        occu, jh, jv, _ = jc.setup_vacancies(seed + k, L, H, pp, bonds, bonds)
        eng.set_disorder(k, p, occu, jh if bonds > 0 else None, jv if bonds > 0 else None)
        eng.set_ladder(k, betas)
        eng.init_spins(k, start, axis)
        models.append(O.Model(L, H, p, occu, jh, jv))
    eng.reset_measurements()
    return eng, models, betas


@pytest.mark.parametrize("L,H", [(8, 4), (10, 10), (4, 2), (16, 6)])
def test_hot_start_is_the_philox_stream(engine_mod, oracle, L, H):
    eng, models, _ = _setup(engine_mod, oracle, L, H, 2, 3, engine_mod.FP64_PLAIN, pp=0.1,
                            conf_base=5)
    for k in range(2):
        for r in range(3):
            exp = oracle.hot_spins_philox(L, H, SEED, 5 + k, r) * models[k].occu
            np.testing.assert_array_equal(eng.spins(k, r), exp)
    eng.close()


@pytest.mark.parametrize("L,H,pp,bonds,flags", [
    (16, 16, 0.0, 0.0, 0),      # quad path
    (8, 4, 0.1, 0.2, 0),        # quad path, vacancies and diluted bonds
    (8, 4, 0.1, 0.2, 16),       # global-memory path (one launch per colour), quad
    (10, 6, 0.1, 0.0, 16),      # global-memory path, per-site
    (10, 10, 0.0, 0.0, 0),      # per-site path (L/2 odd)
    (4, 2, 0.0, 0.0, 0),        # per-site path, doubled J3 and x/y slots (H = 2)
    (12, 6, 0.05, 0.1, 0),      # per-site path with dilution
    (16, 8, 0.05, 0.0, 4),      # per-site path forced on a quad-capable shape
    (24, 24, 0.0, 0.0, 0),      # config-2 lattice
    (32, 32, 0.05, 0.0, 16),    # shape-specialised kernel on lattices in HBM
])
def test_fp64_sweep_bit_identical_to_replay(engine_mod, oracle, L, H, pp, bonds, flags):
    jc = engine_mod
    eng, models, _ = _setup(jc, oracle, L, H, 2, 2, jc.FP64_PLAIN, pp=pp, bonds=bonds,
                            flags=flags)
    for conf in range(2):
        M = models[conf]
        for rep, beta, sweep0, nsw in [(0, 0.11, 37, 3), (1, 0.09, 0, 1), (0, 0.125, 1000, 4)]:
            s = eng.spins(conf, rep).copy()
            got = eng.metro_sweep_fp64(conf, rep, beta, sweep0, nsw)
            flips = M.replay_sweeps(s, beta, SEED, conf, rep, sweep0, nsw)
            assert flips > 0
            np.testing.assert_array_equal(eng.spins(conf, rep), s)
            ints, acc, obs = M.replay_measure(s)
            assert got == (obs[0], obs[1], obs[2], obs[3])
            ref = M.measurement(s)  # the reference's own Measurement of the same configuration
            assert got[0] == ref[0] and got[2] == ref[2] and got[3] == ref[3]
            assert abs(got[1] - ref[1]) < 1e-9  # fixed point: |error| <= N * 2^-33 per site
    eng.close()


@pytest.mark.parametrize("L,H,nconf,nrep,pp,flags", [
    (8, 4, 2, 4, 0.0, 0),
    (8, 8, 3, 5, 0.08, 0),
    (10, 4, 2, 4, 0.0, 0),
    (8, 4, 2, 4, 0.0, 1),   # direct launches instead of the CUDA graph
    (16, 4, 1, 1, 0.0, 0),  # LOCAL sampler: one replica, no swaps
    (24, 24, 1, 2, 0.0, 0),  # shape-specialised FP64 kernel (config-2 lattice)
    (8, 4, 3, 4, 0.1, 16),   # global-memory path
    (32, 32, 1, 2, 0.05, 16),  # shape-specialised kernel on lattices in HBM
    (32, 32, 1, 2, 0.05, 24),  # generic global-memory kernel on the same shape
])
def test_fp64_pt_run_bit_identical_to_replay(engine_mod, oracle, L, H, nconf, nrep, pp, flags):
    jc = engine_mod
    eng, models, betas = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=pp, flags=flags)
    states = []
    for k in range(nconf):
        spins = np.stack([eng.spins(k, r) for r in range(nrep)])
        states.append(oracle.new_pt_state(spins))
    neq, nmess = 7, 12
    eng.run(neq, measure=False, restart_swap_phase=True)
    eng.reset_measurements()
    eng.run(nmess, measure=True, restart_swap_phase=True)
    for k in range(nconf):
        st, M = states[k], models[k]
        M.replay_pt(st, betas, 5, neq, 0, SEED, k, False, 1)
        obs = M.replay_pt(st, betas, 5, nmess, neq, SEED, k, True, 1)
        rat, tor = eng.maps(k)
        np.testing.assert_array_equal(rat, st["rep_at_temp"])
        np.testing.assert_array_equal(tor, st["temp_of_rep"])
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        sums, nm = eng.slot_sums(k)
        np.testing.assert_array_equal(nm, st["nmeas"])
        np.testing.assert_array_equal(sums, st["sums"])
        att, acc, vb = eng.pt_stats(k)
        np.testing.assert_array_equal(att, st["attempts"][:nrep - 1])
        np.testing.assert_array_equal(acc, st["accepts"][:nrep - 1])
        assert vb == int(np.sum(st["visited"] == 3))
        np.testing.assert_array_equal(eng.observables(k), obs)
    eng.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_quad_and_per_site_paths_agree_bitwise(engine_mod, oracle, precision):
    jc = engine_mod
    runs = []
    for flags in (0, jc.FLAG_GENERIC):
        eng, _, _ = _setup(jc, oracle, 16, 8, 2, 4, precision, pp=0.05, bonds=0.1, flags=flags)
        assert eng.config()["sites_per_thread"] == (1 if flags else 4)
        eng.run(10, measure=True)
        runs.append(([eng.spins(k, r) for k in range(2) for r in range(4)],
                     [eng.slot_sums(k)[0] for k in range(2)]))
        eng.close()
    for a, b in zip(runs[0][0], runs[1][0]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(runs[0][1], runs[1][1]):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision,L", [(1, 16), (1, 24), (1, 32), (1, 48), (0, 24), (0, 32)])
def test_specialised_kernels_agree_bitwise(engine_mod, oracle, precision, L):
    """Shape-specialised kernel (every CTA size the autotuner may pick), generic quad kernel
    and per-site kernel give the same spins, observables and running sums."""
    jc = engine_mod
    nts = {16: [128, 64], 24: [448, 224], 32: [1024, 512], 48: [864, 576]}[L] \
        if precision == 1 else \
        {24: [448], 32: [512]}[L]
    runs = []
    for flags, bt in [(jc.FLAG_NO_FIXED, 0), (jc.FLAG_GENERIC, 0), (jc.FLAG_GLOBAL, 0),
                      (jc.FLAG_GLOBAL | jc.FLAG_NO_FIXED, 0)] + \
            [(0, nt) for nt in nts]:
        eng = jc.Engine(L, L, nconf=2, nreplica=3, precision=precision, seed=SEED, flags=flags,
                        block_threads=bt)
        for k in range(2):
            eng.set_disorder(k, jc.disorder(L, L, SEED + k))
            eng.set_ladder(k, _betas(3))
            eng.init_spins(k, jc.START_HOT)
        eng.reset_measurements()
        eng.run(3, measure=True)
        if flags == 0:
            assert eng.config()["block_threads"] == bt
        runs.append(([eng.spins(k, r) for k in range(2) for r in range(3)],
                     eng.slot_sums(-1)[0], eng.observables(-1)))
        eng.close()
    for other in runs[1:]:
        for a, b in zip(runs[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(runs[0][1], other[1])
        np.testing.assert_array_equal(runs[0][2], other[2])


@pytest.mark.parametrize("precision", [0, 1])
def test_mixed_shape_context(engine_mod, oracle, precision):
    """Several lattice shapes in one context (one graph per cycle): every conf evolves exactly as
    in a single-shape context with the same Philox key; FP64 confs also match the replay."""
    jc = engine_mod
    groups = [(8, 4, 2, 3), (10, 6, 1, 2), (16, 16, 2, 4)]
    eng = jc.Engine(groups=groups, precision=precision, seed=SEED)
    models, conf = [], 0
    for L, H, n, r in groups:
        for _ in range(n):
            p = jc.disorder(L, H, SEED + conf)
            occu, _, _, _ = jc.setup_vacancies(SEED + conf, L, H, 0.05)
            eng.set_disorder(conf, p, occu)
            eng.set_ladder(conf, _betas(r))
            eng.init_spins(conf, jc.START_HOT)
            models.append((L, H, r, p, occu))
            conf += 1
    eng.reset_measurements()
    eng.run(4, measure=False)
    eng.reset_measurements()
    eng.run(6, measure=True)
    for k, (L, H, r, p, occu) in enumerate(models):
        single = jc.Engine(L, H, nconf=1, nreplica=r, precision=precision, seed=SEED,
                           conf_base=k)
        single.set_disorder(0, p, occu)
        single.set_ladder(0, _betas(r))
        single.init_spins(0, jc.START_HOT)
        single.reset_measurements()
        single.run(4, measure=False)
        single.reset_measurements()
        single.run(6, measure=True)
        for rep in range(r):
            np.testing.assert_array_equal(eng.spins(k, rep), single.spins(0, rep))
        np.testing.assert_array_equal(eng.slot_sums(k)[0], single.slot_sums(0)[0])
        np.testing.assert_array_equal(eng.maps(k)[0], single.maps(0)[0])
        single.close()
        if precision == 0:
            M = oracle.Model(L, H, p, occu)
            st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) * occu
                                               for q in range(r)]))
            M.replay_pt(st, _betas(r), 5, 4, 0, SEED, k, False, 1)
            M.replay_pt(st, _betas(r), 5, 6, 4, SEED, k, True, 1)
            np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
    eng.close()


def test_large_diluted_lattice_global_path(engine_mod, oracle):
    """L = 96 with 5 % vacancies (config 5 shape) runs on the global-memory path; the kernel's
    observables equal the reference Measurement of the returned configuration."""
    jc = engine_mod
    L = 96
    eng = jc.Engine(L, L, nconf=1, nreplica=2, precision=jc.FP32_BATCHED, seed=SEED)
    p = jc.disorder(L, L, SEED)
    occu, _, _, nimp = jc.setup_vacancies(SEED, L, L, 0.05)
    assert 0.04 < nimp / L ** 3 < 0.06
    eng.set_disorder(0, p, occu)
    eng.set_ladder(0, _betas(2))
    eng.init_spins(0, jc.START_HOT)
    eng.reset_measurements()
    eng.run(2, measure=True)
    M = oracle.Model(L, L, p, occu)
    obs = eng.observables(0)
    for rep in range(2):
        s = eng.spins(0, rep)
        assert (s[occu == 0] == 0).all() and set(np.unique(s[occu == 1])) <= {-1, 1}
        ref = M.measurement(s)
        assert obs[rep, 0] == ref[0] and obs[rep, 2] == ref[2] and obs[rep, 3] == ref[3]
        assert abs(obs[rep, 1] - ref[1]) < 1e-5  # FP32 field per site
        assert obs[rep, 4] == M.nbar(s)
    eng.close()


def test_fp32_decision_mismatch_rate(engine_mod, oracle):
    jc = engine_mod
    eng, _, _ = _setup(jc, oracle, 16, 16, 4, 8, jc.FP32_BATCHED)
    eng.run(20, measure=False)
    att, mis = eng.audit_fp32(20)
    assert att == 4 * 8 * 16 ** 3 * 20
    rate = mis / att
    print(f"FP32 vs FP64 flip-decision mismatch rate: {rate:.3e} ({mis}/{att})")
    assert rate < 1e-4
    eng.close()


def test_fp32_observables_match_fp64(engine_mod, oracle):
    """Same disorder and streams: per-conf thermal averages of FP32 and FP64 differ only by
    statistical noise (the two trajectories decorrelate after the first flipped decision).  Each
    observable's FP32 - FP64 difference at each temperature slot, in units of its standard error
    over the configurations, is "within 2 sigma" in the statistical sense: at most 15 % of the
    48 z-scores beyond 2 (5.7 % expected for 23 degrees of freedom; the observables are
    correlated) and none beyond 4."""
    jc = engine_mod
    nconf, nrep, L, nmess = 24, 6, 8, 1500
    names = ("absmag", "mag2", "en", "en2", "strx_abs", "stry_abs", "nbar", "nbar2")
    cols = [jc.SUM_FIELDS.index(n) for n in names]
    res = {}
    for prec in (jc.FP64_PLAIN, jc.FP32_BATCHED):
        eng, _, betas = _setup(jc, oracle, L, L, nconf, nrep, prec)
        eng.run(300, measure=False)
        eng.reset_measurements()
        eng.run(nmess, measure=True)
        res[prec] = np.array([eng.slot_sums(k)[0][:, cols] / nmess for k in range(nconf)])
        eng.close()
    d = res[jc.FP32_BATCHED] - res[jc.FP64_PLAIN]  # (nconf, nrep, observable)
    se = d.std(axis=0, ddof=1) / np.sqrt(nconf)
    z = np.abs(d.mean(axis=0)) / (se + 1e-300)
    for j, n in enumerate(names):
        print(f"FP32 - FP64 {n:9s} |z| by slot:", " ".join(f"{v:4.2f}" for v in z[:, j]))
    assert (z > 2).mean() <= 0.15, z
    assert z.max() < 4, z


def test_invalid_calls_fail_cleanly(engine_mod, oracle):
    jc = engine_mod
    eng = jc.Engine(8, 4, nconf=2, nreplica=3, precision=jc.FP32_BATCHED)
    with pytest.raises(jc.J1J2CError) as e:
        eng.run(1)
    assert e.value.code == jc.ESTATE
    with pytest.raises(jc.J1J2CError):
        eng.set_disorder(5, np.zeros(8 * 8 * 4))
    with pytest.raises(jc.J1J2CError) as e:
        eng.init_spins(0)
    assert e.value.code == jc.ESTATE
    eng.set_disorder(0, np.zeros(8 * 8 * 4))
    with pytest.raises(jc.J1J2CError):
        eng.init_spins(0, spins=np.zeros((3, 256), np.int8))
    with pytest.raises(jc.J1J2CError):
        eng.set_ladder(0, np.array([1.0, np.nan, 2.0]))
    eng.close()


def test_cluster_path_fp64_bit_identical(engine_mod, oracle):
    """A lattice too large for one CTA's shared memory (64^3: 256 KiB of spins) runs on the
    thread-block-cluster kernel (4 CTAs of 64 KiB, distributed shared memory; a fixed CTA size
    keeps the autotuner from switching to the global path); FP64 with vacancies and diluted bonds
    equals the oracle's replay bit for bit."""
    jc = engine_mod
    L = H = 64
    eng, models, betas = _setup(jc, oracle, L, H, 1, 2, jc.FP64_PLAIN, pp=0.05, bonds=0.1,
                                block_threads=512)
    cfg = eng.config()
    assert cfg["block_threads"] == 512 and cfg["smem_bytes"] == L * L * H // 4
    st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, 0, q) * models[0].occu
                                       for q in range(2)]))
    eng.run(2, measure=False)
    eng.reset_measurements()
    eng.run(2, measure=True)
    M = models[0]
    M.replay_pt(st, betas, 5, 2, 0, SEED, 0, False, 1)
    M.replay_pt(st, betas, 5, 2, 2, SEED, 0, True, 1)
    for r in range(2):
        np.testing.assert_array_equal(eng.spins(0, r), st["spins"][r])
    np.testing.assert_array_equal(eng.slot_sums(0)[0], st["sums"])
    np.testing.assert_array_equal(eng.maps(0)[0], st["rep_at_temp"])
    eng.close()


@pytest.mark.parametrize("pp,bonds", [(0.05, 0.0), (0.0, 0.1)])
def test_cluster_path_fp32_equals_global_path(engine_mod, oracle, pp, bonds):
    """FP32, 96 x 96 x 32 (the cluster kernel, 4 CTAs per lattice) against the one-launch-per-
    colour global-memory kernel: bitwise equal spins, sums and observables."""
    jc = engine_mod
    out = []
    for flags in (0, jc.FLAG_GLOBAL):
        eng, _, _ = _setup(jc, oracle, 96, 32, 2, 2, jc.FP32_BATCHED, pp=pp, bonds=bonds,
                           flags=flags, block_threads=512)
        eng.run(3, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(2)],
                    [eng.slot_sums(k)[0] for k in range(2)], eng.observables(-1),
                    eng.config()["smem_bytes"]))
        eng.close()
    assert out[0][3] == 96 * 96 * 32 // 4 and out[1][3] == 0
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(out[0][1], out[1][1]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("precision,nrep", [(0, 4), (1, 4), (1, 2), (1, 3)])
def test_hbm_kernel_replicas_per_thread(engine_mod, oracle, precision, nrep):
    """The HBM kernel with 4, 2 or 1 replicas per thread (chosen from the replica count under
    the global-memory flag) against the generic shared-memory kernel: bitwise equal, 32^3 with
    vacancies."""
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_NO_FIXED, jc.FLAG_GLOBAL):
        eng, _, _ = _setup(jc, oracle, 32, 32, 2, nrep, precision, pp=0.05, flags=flags)
        eng.run(2, measure=False)
        eng.run(3, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(nrep)],
                    eng.slot_sums(-1)[0], eng.observables(-1), eng.config()["smem_bytes"]))
        eng.close()
    assert out[0][3] > 0 and out[1][3] == 0
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("L,pp", [(32, 0.0), (32, 0.05), (24, 0.05), (16, 0.05)])
def test_streaming_kernel_equals_per_lattice_kernel(engine_mod, oracle, L, pp):
    """FP32: the streaming form (one CTA per SM through a range of lattices, spins double-
    buffered by bulk copies, the field reloaded where the range crosses a configuration) against
    one CTA per lattice: bitwise equal spins, sums and observables, 320 lattices."""
    jc = engine_mod
    nconf, nrep = 10, 32
    out = []
    for flags, bt in ((0, {32: 1024, 24: 448, 16: 128}[L]), (jc.FLAG_STREAM, 0)):
        eng, _, _ = _setup(jc, oracle, L, L, nconf, nrep, jc.FP32_BATCHED, pp=pp, flags=flags,
                           block_threads=bt)
        eng.run(2, measure=False)
        eng.run(2, measure=True)
        out.append(([eng.spins(k, r) for k in range(nconf) for r in range(nrep)],
                    eng.slot_sums(-1)[0], eng.observables(-1)))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_hbm_kernel_L96_fp64_bit_identical_to_replay(engine_mod, oracle):
    """96^3 with 5 % vacancies (the reference's largest configuration) through the shape-
    specialised kernel that keeps lattices in HBM: spins, maps and running sums equal the replay."""
    jc = engine_mod
    L, nrep = 96, 2
    eng, models, betas = _setup(jc, oracle, L, L, 1, nrep, jc.FP64_PLAIN, pp=0.05,
                                flags=jc.FLAG_GLOBAL)
    assert eng.config()["smem_bytes"] == 0 and eng.config()["block_threads"] == 256
    st = oracle.new_pt_state(np.stack([eng.spins(0, r) for r in range(nrep)]))
    eng.run(1, measure=False, restart_swap_phase=True)
    eng.reset_measurements()
    eng.run(2, measure=True, restart_swap_phase=True)
    M = models[0]
    M.replay_pt(st, betas, 5, 1, 0, SEED, 0, False, 1)
    obs = M.replay_pt(st, betas, 5, 2, 1, SEED, 0, True, 1)
    for r in range(nrep):
        np.testing.assert_array_equal(eng.spins(0, r), st["spins"][r])
    np.testing.assert_array_equal(eng.slot_sums(0)[0], st["sums"])
    np.testing.assert_array_equal(eng.maps(0)[0], st["rep_at_temp"])
    np.testing.assert_array_equal(eng.observables(0), obs)
    eng.close()


def test_hbm_kernel_L96_fp32_equals_other_paths(engine_mod, oracle):
    """FP32 96^3 with vacancies: the shape-specialised HBM kernel (CTAs of 256, 128 and 512
    threads), the generic global-memory kernel and the default choice (thread-block cluster or
    HBM kernel, whichever the autotuner keeps) give bitwise equal spins, sums and
    observables."""
    jc = engine_mod
    out = []
    for flags, bt in ((jc.FLAG_GLOBAL, 0), (jc.FLAG_GLOBAL, 128), (jc.FLAG_GLOBAL, 512),
                      (jc.FLAG_GLOBAL | jc.FLAG_NO_FIXED, 0), (0, 0)):
        eng, _, _ = _setup(jc, oracle, 96, 96, 1, 3, jc.FP32_BATCHED, pp=0.05, flags=flags,
                           block_threads=bt)
        eng.run(2, measure=True)
        if bt:
            assert eng.config()["block_threads"] == bt
        out.append(([eng.spins(0, r) for r in range(3)], eng.slot_sums(0)[0],
                    eng.observables(-1)))
        eng.close()
    for other in out[1:]:
        for a, b in zip(out[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(out[0][1], other[1])
        np.testing.assert_array_equal(out[0][2], other[2])


@pytest.mark.parametrize("L,H,nconf,nrep,pp", [(24, 24, 1, 16, 0.0), (16, 16, 1, 1, 0.05),
                                                (32, 8, 2, 2, 0.1)])
def test_small_batch_cluster_path_fp64_bit_identical(engine_mod, oracle, L, H, nconf, nrep, pp):
    """Small batches may run one lattice over a cluster of up to 16 CTAs (the autotuner's
    small-batch choice; flag 64 pins the largest cluster): FP64 equals the replay bit for bit,
    including the PT SERIAL configuration (24^3, 16 replicas) and a single-lattice LOCAL-style run."""
    jc = engine_mod
    eng, models, betas = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=pp,
                                flags=jc.FLAG_CLUSTER)
    assert eng.config()["block_threads"] == 512
    eng.run(2, measure=False)
    eng.reset_measurements()
    eng.run(3, measure=True)
    for k in range(nconf):
        st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) *
                                           models[k].occu for q in range(nrep)]))
        models[k].replay_pt(st, betas, 5, 2, 0, SEED, k, False, 1)
        models[k].replay_pt(st, betas, 5, 3, 2, SEED, k, True, 1)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
    eng.close()


@pytest.mark.parametrize("L,H,nconf,nrep,pp", [(16, 16, 1, 1, 0.05), (24, 24, 1, 4, 0.0),
                                                (32, 8, 2, 2, 0.1)])
def test_small_batch_site_cluster_fp64_bit_identical(engine_mod, oracle, L, H, nconf, nrep, pp):
    """One site per thread over a thread-block cluster (flags CLUSTER + GENERIC; a small-batch
    choice of the autotuner): FP64 equals the replay bit for bit, the LOCAL shape included."""
    jc = engine_mod
    eng, models, betas = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=pp,
                                flags=jc.FLAG_CLUSTER | jc.FLAG_GENERIC)
    cfg = eng.config()
    assert cfg["sites_per_thread"] == 1 and 0 < cfg["smem_bytes"] < L * L * H
    eng.run(2, measure=False)
    eng.reset_measurements()
    eng.run(3, measure=True)
    for k in range(nconf):
        st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) *
                                           models[k].occu for q in range(nrep)]))
        models[k].replay_pt(st, betas, 5, 2, 0, SEED, k, False, 1)
        obs = models[k].replay_pt(st, betas, 5, 3, 2, SEED, k, True, 1)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
        np.testing.assert_array_equal(eng.observables(k), obs)
    eng.close()


def test_small_batch_site_cluster_fp32_bitwise(engine_mod, oracle):
    """FP32: one site per thread over a cluster equals the shared-memory kernels bit for bit."""
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_NO_FIXED, jc.FLAG_CLUSTER | jc.FLAG_GENERIC):
        eng, _, _ = _setup(jc, oracle, 32, 16, 2, 3, jc.FP32_BATCHED, pp=0.05, flags=flags)
        eng.run(4, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(3)],
                    eng.slot_sums(-1)[0], eng.observables(-1), eng.config()))
        eng.close()
    assert out[1][3]["sites_per_thread"] == 1
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_small_batch_cluster_path_fp32_bitwise(engine_mod, oracle):
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_CLUSTER, jc.FLAG_NO_FIXED):
        eng, _, _ = _setup(jc, oracle, 32, 32, 2, 3, jc.FP32_BATCHED, pp=0.05, flags=flags)
        eng.run(3, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(3)], eng.slot_sums(-1)[0],
                    eng.observables(-1)))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


def test_non_integer_couplings(engine_mod, oracle):
    """J2 = -0.7, J3 = 1.3: the shape-specialised FP32 kernels form J3*Zs + J2*D in integer
    arithmetic and so take integer J2, J3 only; here the FP32 form runs the generic kernels,
    whose variants agree bit for bit, and the FP64 form (shape-specialised kernel, any
    couplings) equals the oracle's replay bit for bit."""
    jc = engine_mod
    L, nrep, J2, J3 = 32, 3, -0.7, 1.3
    betas = _betas(nrep)
    out = []
    for flags in (0, jc.FLAG_GENERIC, jc.FLAG_GLOBAL):
        eng = jc.Engine(L, L, nconf=2, nreplica=nrep, precision=jc.FP32_BATCHED, seed=SEED,
                        flags=flags, J2=J2, J3=J3)
        for k in range(2):
            eng.set_disorder(k, jc.disorder(L, L, SEED + k))
            eng.set_ladder(k, betas)
            eng.init_spins(k, jc.START_HOT)
        eng.reset_measurements()
        eng.run(3, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(nrep)],
                    eng.slot_sums(-1)[0], eng.observables(-1)))
        eng.close()
    for other in out[1:]:
        for a, b in zip(out[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(out[0][1], other[1])
        np.testing.assert_array_equal(out[0][2], other[2])
    p = jc.disorder(L, L, SEED)
    eng = jc.Engine(L, L, nconf=1, nreplica=nrep, precision=jc.FP64_PLAIN, seed=SEED, J2=J2, J3=J3)
    eng.set_disorder(0, p)
    eng.set_ladder(0, betas)
    eng.init_spins(0, jc.START_HOT)
    eng.reset_measurements()
    st = oracle.new_pt_state(np.stack([eng.spins(0, r) for r in range(nrep)]))
    eng.run(4, measure=True)
    M = oracle.Model(L, L, p, J2=J2, J3=J3)
    obs = M.replay_pt(st, betas, 5, 4, 0, SEED, 0, True, 1)
    for r in range(nrep):
        np.testing.assert_array_equal(eng.spins(0, r), st["spins"][r])
    np.testing.assert_array_equal(eng.slot_sums(0)[0], st["sums"])
    np.testing.assert_array_equal(eng.observables(0), obs)
    eng.close()


@pytest.mark.parametrize("L,pp,nrep", [(32, 0.0, 32), (32, 0.05, 8), (24, 0.05, 24),
                                        (16, 0.05, 16)])
def test_pair_kernel_equals_per_lattice_kernel(engine_mod, oracle, L, pp, nrep):
    """FP32: two replicas of one configuration per CTA (their lattices behind one shared copy of
    the field, each quad position's field operands loaded once for both) against one CTA per
    lattice: bitwise equal spins, sums and observables, over cycles with replica exchanges."""
    jc = engine_mod
    nconf = 3
    out = []
    for flags, bt in ((0, {32: 512, 24: 448, 16: 128}[L]), (jc.FLAG_PAIRS, 0)):
        eng, _, _ = _setup(jc, oracle, L, L, nconf, nrep, jc.FP32_BATCHED, pp=pp, flags=flags,
                           block_threads=bt)
        eng.run(2, measure=False)
        eng.run(3, measure=True)
        cfg = eng.config()
        out.append(([eng.spins(k, r) for k in range(nconf) for r in range(nrep)],
                    eng.slot_sums(-1)[0], eng.observables(-1), cfg))
        eng.close()
    n = L ** 3
    assert out[1][3]["smem_bytes"] == 2 * n + 4 * n, out[1][3]
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("pp,wolff", [(0.0, False), (0.05, False), (0.05, True)])
def test_multi_shape_launch_equals_single_shape_contexts(engine_mod, oracle, pp, wolff):
    """Lattice shapes L = 16, 24, 32, 48 in one context swept by one persistent launch (flag
    8192: a CTA per SM takes tiles of R replicas of one configuration from one queue) equal
    single-shape contexts with the same Philox keys bit for bit: spins, running sums, maps and
    observables over cycles with replica exchanges (and Wolff updates)."""
    jc = engine_mod
    groups = [(16, 16, 2, 16), (24, 24, 1, 24), (32, 32, 2, 32), (48, 48, 1, 48)]
    flags = jc.FLAG_MULTI | (jc.FLAG_WOLFF if wolff else 0)
    eng = jc.Engine(groups=groups, precision=jc.FP32_BATCHED, seed=SEED, flags=flags)
    confs, conf = [], 0
    for L, H, n, r in groups:
        for _ in range(n):
            p = jc.disorder(L, H, SEED + conf)
            occu = jc.setup_vacancies(SEED + conf, L, H, pp)[0] if pp > 0 else None
            eng.set_disorder(conf, p, occu)
            eng.set_ladder(conf, _betas(r))
            eng.init_spins(conf, jc.START_HOT)
            confs.append((L, H, r, p, occu))
            conf += 1
    eng.reset_measurements()
    eng.run(2, measure=False)
    eng.reset_measurements()
    eng.run(3, measure=True)
    cfg = eng.config()
    assert cfg["block_threads"] == 512 and cfg["smem_bytes"] == 2 * 32 ** 3 + 4 * 32 ** 3, cfg
    for k, (L, H, r, p, occu) in enumerate(confs):
        single = jc.Engine(L, H, nconf=1, nreplica=r, precision=jc.FP32_BATCHED, seed=SEED,
                           conf_base=k, flags=jc.FLAG_WOLFF if wolff else 0)
        single.set_disorder(0, p, occu)
        single.set_ladder(0, _betas(r))
        single.init_spins(0, jc.START_HOT)
        single.reset_measurements()
        single.run(2, measure=False)
        single.reset_measurements()
        single.run(3, measure=True)
        for rep in range(r):
            np.testing.assert_array_equal(eng.spins(k, rep), single.spins(0, rep))
        np.testing.assert_array_equal(eng.slot_sums(k)[0], single.slot_sums(0)[0])
        np.testing.assert_array_equal(eng.maps(k)[0], single.maps(0)[0])
        np.testing.assert_array_equal(eng.observables(k), single.observables(0))
        single.close()
    eng.close()


@pytest.mark.parametrize("L,H,nconf,nrep,pp,ptswapever", [(16, 16, 1, 1, 0.05, 1),
                                                           (24, 24, 1, 16, 0.0, 5),
                                                           (32, 8, 2, 2, 0.1, 5)])
def test_cooperative_small_batch_fp64_bit_identical(engine_mod, oracle, L, H, nconf, nrep, pp,
                                                    ptswapever):
    """Small batches with every colour phase, sweep and the observables of a cycle in one
    cooperative launch (flag 16384; grid barriers between the phases): FP64 equals the replay
    bit for bit, the LOCAL shape (one lattice, one sweep per cycle) and the PT configuration's
    shape included."""
    jc = engine_mod
    betas = _betas(nrep) if nrep > 1 else np.array([1.0 / 9.5])
    eng, models, _ = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=pp,
                            flags=jc.FLAG_COOP, ptswapever=ptswapever, betas=betas)
    eng.run(3, measure=False)
    eng.reset_measurements()
    eng.run(4, measure=True)
    assert eng.config()["smem_bytes"] == 0 and eng.config()["block_threads"] == 64
    for k in range(nconf):
        st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) *
                                           models[k].occu for q in range(nrep)]))
        models[k].replay_pt(st, betas, ptswapever, 3, 0, SEED, k, False, 1)
        obs = models[k].replay_pt(st, betas, ptswapever, 4, 3, SEED, k, True, 1)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
        np.testing.assert_array_equal(eng.observables(k), obs)
    eng.close()


def test_cooperative_small_batch_fp32_bitwise(engine_mod, oracle):
    """FP32: the cooperative form equals the generic shared-memory kernels bit for bit."""
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_NO_FIXED, jc.FLAG_COOP):
        eng, _, _ = _setup(jc, oracle, 32, 16, 2, 3, jc.FP32_BATCHED, pp=0.05, flags=flags)
        eng.run(4, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(3)],
                    eng.slot_sums(-1)[0], eng.observables(-1)))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("L,H,nconf,nrep,pp,bonds,ptswapever,cs", [
    (16, 16, 1, 1, 0.05, 0.0, 1, 0), (16, 16, 1, 1, 0.0, 0.0, 1, 4), (16, 16, 1, 2, 0.05, 0.0, 1, 8),
    (24, 24, 1, 16, 0.0, 0.0, 5, 0), (24, 24, 1, 4, 0.05, 0.0, 5, 8), (24, 24, 2, 2, 0.0, 0.0, 5, 4),
    (8, 4, 2, 2, 0.1, 0.2, 5, 0)])
def test_replicated_cluster_fp64_bit_identical(engine_mod, oracle, monkeypatch, L, H, nconf, nrep,
                                               pp, bonds, ptswapever, cs):
    """Small batches with the lattice replicated in every CTA of a thread-block cluster (flag
    32768; each CTA updates 1/cs of every colour and copies it into its peers' shared memory):
    FP64 equals the replay bit for bit, the LOCAL shape (one lattice, one sweep per cycle), the PT
    configuration's shape and diluted bonds included.  L = 16 and 24 run the compile-time-shape
    kernel with 16 (the pin's default), 8 or 4 CTAs per lattice; 8 x 4 with diluted bonds the
    runtime-shape one."""
    jc = engine_mod
    if cs:
        monkeypatch.setenv("J1J2C_REPLICA_CS", str(cs))
    betas = _betas(nrep) if nrep > 1 else np.array([1.0 / 9.5])
    eng, models, _ = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=pp, bonds=bonds,
                            flags=jc.FLAG_REPLICA, ptswapever=ptswapever, betas=betas)
    eng.run(3, measure=False)
    eng.reset_measurements()
    eng.run(4, measure=True)
    cfg = eng.config()
    assert cfg["sites_per_thread"] == 1 and cfg["smem_bytes"] > L * L * H
    for k in range(nconf):
        st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) *
                                           models[k].occu for q in range(nrep)]))
        models[k].replay_pt(st, betas, ptswapever, 3, 0, SEED, k, False, 1)
        obs = models[k].replay_pt(st, betas, ptswapever, 4, 3, SEED, k, True, 1)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
        np.testing.assert_array_equal(eng.observables(k), obs)
    eng.close()


def test_replicated_cluster_fp32_and_flip_counts_bitwise(engine_mod, oracle):
    """FP32 with vacancies: the replicated-lattice cluster form equals the generic shared-memory
    kernels bit for bit, flip counts included."""
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_NO_FIXED, jc.FLAG_REPLICA):
        eng, _, _ = _setup(jc, oracle, 32, 16, 2, 3, jc.FP32_BATCHED, pp=0.05, flags=flags)
        eng.set_diagnostics(flip_counts=True)
        eng.run(4, measure=True)
        out.append(([eng.spins(k, r) for k in range(2) for r in range(3)],
                    eng.slot_sums(-1)[0], eng.observables(-1),
                    [eng.flip_counts(k) for k in range(2)]))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])
    for a, b in zip(out[0][3], out[1][3]):
        np.testing.assert_array_equal(a, b)


def test_enqueue_then_sync_equals_run(engine_mod, oracle):
    """Cycles queued with j1j2c_enqueue (no wait) and collected with j1j2c_sync give exactly the
    state j1j2c_run gives (FP64, equal to the replay too)."""
    jc = engine_mod
    L, H, nconf, nrep = 16, 8, 2, 4
    out = []
    for mode in ("run", "enqueue"):
        eng, models, betas = _setup(jc, oracle, L, H, nconf, nrep, jc.FP64_PLAIN, pp=0.05)
        if mode == "run":
            eng.run(3, measure=True)
        else:
            eng.enqueue(1, measure=True, restart_swap_phase=True)
            eng.enqueue(2, measure=True, restart_swap_phase=False)
            eng.sync()
        out.append(([eng.spins(k, r) for k in range(nconf) for r in range(nrep)],
                    eng.slot_sums(-1)[0], eng.maps(0)[0]))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][2], out[1][2])

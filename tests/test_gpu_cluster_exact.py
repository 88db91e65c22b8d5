"""GPU: Wolff cluster update (bit-identical to the oracle's restatement, inside and outside PT
cycles) and exact enumeration (against a CPU enumeration with the reference Measurement, and
as the oracle of the sampled Metropolis / PT / Wolff averages on 4 x 4 x 2)."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 3


def _betas(n, tmin=8.0, tmax=11.5):
    from oracle import oracle as O
    return 1.0 / O.ladder(n, tmin, tmax)


def _engine(jc, L, H, nconf, nrep, precision, flags=0, pp=0.0, bonds=0.0, betas=None,
            same_disorder=False):
    eng = jc.Engine(L, H, nconf=nconf, nreplica=nrep, precision=precision, seed=SEED,
                    flags=flags)
    betas = _betas(nrep) if betas is None else betas
    dis = []
    for k in range(nconf):
        sd = SEED if same_disorder else SEED + k
        p = jc.disorder(L, H, sd)
        occu, jh, jv, _ = jc.setup_vacancies(sd, L, H, pp, bonds, bonds)
        eng.set_disorder(k, p, occu, jh if bonds else None, jv if bonds else None)
        eng.set_ladder(k, betas)
        eng.init_spins(k, jc.START_HOT)
        dis.append((p, occu, jh, jv))
    eng.reset_measurements()
    return eng, dis, betas


# Forms: flags 0 / 16 the seed-cluster growth (default), 8 the shared-memory slab labelling,
# 4 the per-site global labelling; 128 / 256 the growth over a cluster of 2 / 4 CTAs per lattice,
# 384 two CTAs for the coldest quarter of the slots and one for the rest (two launches), 2048 the
# growth from bond activations decided beforehand on every SM (the quad store and, with L/2 odd,
# the byte stores), 65536 the level-free growth (a work queue instead of breadth-first levels).  Slab shapes: one slab per lattice (8 x 4), several slabs with
# the +z boundary merge (48^3: 3 slabs of 16 planes; 96 x 8: 2 slabs of 4), one-CTA-per-SM slabs
# (160 x 4: 2 slabs of 2 planes), no slab fits (200 x 4: the per-site form is used).
@pytest.mark.parametrize("L,H,pp,bonds,flags", [(8, 4, 0.1, 0.2, 0), (10, 6, 0.0, 0.0, 0),
                                                 (4, 2, 0.0, 0.0, 0), (8, 8, 0.05, 0.0, 16),
                                                 (8, 4, 0.1, 0.2, 4), (8, 4, 0.1, 0.2, 8),
                                                 (48, 48, 0.05, 0.0, 0), (48, 48, 0.05, 0.0, 8),
                                                 (96, 8, 0.1, 0.2, 0), (96, 8, 0.1, 0.2, 8),
                                                 (160, 4, 0.0, 0.0, 8), (200, 4, 0.05, 0.0, 8),
                                                 (2, 2, 0.0, 0.0, 0), (8, 4, 0.1, 0.2, 128),
                                                 (48, 48, 0.05, 0.0, 128),
                                                 (96, 8, 0.1, 0.2, 256), (10, 6, 0.0, 0.0, 256),
                                                 (48, 48, 0.05, 0.0, 384),
                                                 (8, 4, 0.1, 0.2, 2048), (10, 6, 0.0, 0.0, 2048),
                                                 (48, 48, 0.05, 0.0, 2048),
                                                 (96, 8, 0.1, 0.2, 2048), (2, 2, 0.0, 0.0, 2048),
                                                 (8, 4, 0.1, 0.2, 65536),
                                                 (10, 6, 0.0, 0.0, 65536),
                                                 (4, 2, 0.0, 0.0, 65536), (2, 2, 0.0, 0.0, 65536),
                                                 (48, 48, 0.05, 0.0, 65536),
                                                 (96, 8, 0.1, 0.2, 65536)])
def test_wolff_step_bit_identical(engine_mod, oracle, L, H, pp, bonds, flags):
    jc = engine_mod
    eng, dis, betas = _engine(jc, L, H, 2, 3, jc.FP64_PLAIN, flags, pp, bonds)
    eng.run(3, measure=False)
    before = {(k, r): eng.spins(k, r).copy() for k in range(2) for r in range(3)}
    tors = [eng.maps(k)[1] for k in range(2)]
    sizes = eng.wolff()
    total = 0
    for k in range(2):
        p, occu, jh, jv = dis[k]
        M = oracle.Model(L, H, p, occu, jh if bonds else None, jv if bonds else None)
        for r in range(3):
            s = before[(k, r)].copy()
            n = M.wolff_step(s, betas[tors[k][r]], SEED, k, r, 3)
            np.testing.assert_array_equal(eng.spins(k, r), s)
            assert sizes[3 * k + r] == n
            total += n
    assert total > 0
    eng.close()


@pytest.mark.parametrize("nconf,flags", [(40, 0), (80, 0), (40, 128), (40, 256), (80, 384),
                                         (80, 2048), (80, 65536)])
def test_wolff_growth_many_lattices(engine_mod, oracle, nconf, flags):
    """More lattices than SMs (160 and 320 lattices: two and three waves of growth CTAs, coldest
    slots first): the flipped clusters equal the oracle's in the first, middle and last
    configuration."""
    jc = engine_mod
    L, H, nrep = 16, 16, 4
    eng, dis, betas = _engine(jc, L, H, nconf, nrep, jc.FP64_PLAIN, flags, 0.05)
    eng.run(2, measure=False)
    check = (0, nconf // 2, nconf - 1)
    before = {(k, r): eng.spins(k, r).copy() for k in check for r in range(nrep)}
    tors = {k: eng.maps(k)[1] for k in check}
    sizes = eng.wolff()
    assert len(sizes) == nconf * nrep and sizes.sum() > 0
    for k in check:
        p, occu, _, _ = dis[k]
        M = oracle.Model(L, H, p, occu)
        for r in range(nrep):
            s = before[(k, r)].copy()
            n = M.wolff_step(s, betas[tors[k][r]], SEED, k, r, 2)
            np.testing.assert_array_equal(eng.spins(k, r), s)
            assert sizes[nrep * k + r] == n
    eng.close()


@pytest.mark.parametrize("L,H,pp,bonds", [(96, 8, 0.1, 0.2), (48, 48, 0.05, 0.0),
                                          (32, 32, 0.0, 0.0), (160, 4, 0.05, 0.0)])
def test_wolff_fp32_forms_agree(engine_mod, oracle, L, H, pp, bonds):
    """FP32: the seed-cluster growth, the shared-memory slab labelling and the per-site global
    union-find flip exactly the same clusters (same activated bonds, same component of the seed),
    after sweeps and over several cycles."""
    jc = engine_mod
    out = []
    for flags in (jc.FLAG_WOLFF, jc.FLAG_WOLFF | jc.FLAG_NO_FIXED, jc.FLAG_WOLFF | jc.FLAG_GENERIC,
                  jc.FLAG_WOLFF | jc.FLAG_WOLFF_CS2, jc.FLAG_WOLFF | jc.FLAG_WOLFF_CS4,
                  jc.FLAG_WOLFF | jc.FLAG_WOLFF_CS2 | jc.FLAG_WOLFF_CS4,
                  jc.FLAG_WOLFF | jc.FLAG_WOLFF_BITS, jc.FLAG_WOLFF | jc.FLAG_WOLFF_ASYNC):
        eng, _, _ = _engine(jc, L, H, 2, 3, jc.FP32_BATCHED, flags, pp, bonds)
        sizes = [eng.wolff().copy()]
        eng.run(3, measure=True)
        sizes.append(eng.cluster_sizes().copy())
        out.append(([eng.spins(k, r).copy() for k in range(2) for r in range(3)], sizes))
        eng.close()
    for other in out[1:]:
        for a, b in zip(out[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        for a, b in zip(out[0][1], other[1]):
            np.testing.assert_array_equal(a, b)
    assert sum(int(x.sum()) for x in out[0][1]) > 0


@pytest.mark.parametrize("nrep", [4, 8])
def test_wolff_inside_pt_cycles(engine_mod, oracle, nrep):
    """PT cycles with a Wolff update first (the CTAs-per-lattice tuner runs at the first cycle;
    with 8 replicas it also times the split over two launches) equal the replay."""
    jc = engine_mod
    L, H = 8, 4
    eng, dis, betas = _engine(jc, L, H, 2, nrep, jc.FP64_PLAIN, jc.FLAG_WOLFF, 0.05)
    states = [oracle.new_pt_state(np.stack([eng.spins(k, r) for r in range(nrep)]))
              for k in range(2)]
    eng.run(6, measure=True)
    for k in range(2):
        p, occu, _, _ = dis[k]
        M = oracle.Model(L, H, p, occu)
        st = states[k]
        for cyc in range(6):
            for r in range(nrep):
                s = st["spins"][r].copy()
                M.wolff_step(s, betas[st["temp_of_rep"][r]], SEED, k, r, cyc)
                st["spins"][r] = s
            M.replay_pt(st, betas, 5, 1, cyc, SEED, k, True, 1 if cyc % 2 == 0 else 2)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
    assert (eng.cluster_sizes() >= 0).all()
    eng.close()


@pytest.mark.parametrize("extra", ["split", "tuned", "split_bits", "split_async", "split3",
                                   "split4", "split5"])
def test_split_wolff_sweeps_bit_identical(engine_mod, oracle, extra, monkeypatch):
    """Lattices in HBM (the one-launch-per-colour kernel; L = 32 is its cross-check shape) with a
    Wolff update per cycle: the Wolff update and sweeps of the coldest slots and of the others
    on two streams, each sweep launch finding its lattices through the temperature map (flag
    1024 pins the split at a quarter of the slots, with flag 2048 the cold slots' bonds decided
    beforehand, with flag 65536 the one-CTA growths level-free, with J1J2C_SPLIT=2,5 three
    ranges on three streams, with 1,3,6 four, with 1,2,4,6 five; unpinned the tuner times the
    candidates on equilibrated scratch lattices), equal the replay bit for bit over cycles with
    replica exchanges."""
    jc = engine_mod
    pins = {"split3": "2,5", "split4": "1,3,6", "split5": "1,2,4,6"}
    if extra in pins:
        monkeypatch.setenv("J1J2C_SPLIT", pins[extra])
    L, H, nconf, nrep, ncyc = 32, 32, 2, 8, 3
    flags = jc.FLAG_WOLFF | jc.FLAG_GLOBAL | {"split": jc.FLAG_WOLFF_SPLIT, "tuned": 0,
                                              "split_bits": jc.FLAG_WOLFF_SPLIT |
                                              jc.FLAG_WOLFF_BITS,
                                              "split_async": jc.FLAG_WOLFF_SPLIT |
                                              jc.FLAG_WOLFF_ASYNC,
                                              "split3": jc.FLAG_WOLFF_SPLIT,
                                              "split4": jc.FLAG_WOLFF_SPLIT,
                                              "split5": jc.FLAG_WOLFF_SPLIT}[extra]
    eng, dis, betas = _engine(jc, L, H, nconf, nrep, jc.FP64_PLAIN, flags, 0.05)
    states = [oracle.new_pt_state(np.stack([eng.spins(k, r) for r in range(nrep)]))
              for k in range(nconf)]
    eng.run(ncyc, measure=True, restart_swap_phase=True)
    assert eng.config()["smem_bytes"] == 0
    for k in range(nconf):
        p, occu, _, _ = dis[k]
        M = oracle.Model(L, H, p, occu)
        st = states[k]
        for cyc in range(ncyc):
            for r in range(nrep):
                s = st["spins"][r].copy()
                M.wolff_step(s, betas[st["temp_of_rep"][r]], SEED, k, r, cyc)
                st["spins"][r] = s
            M.replay_pt(st, betas, 5, 1, cyc, SEED, k, True, 1 if cyc % 2 == 0 else 2)
        for r in range(nrep):
            np.testing.assert_array_equal(eng.spins(k, r), st["spins"][r])
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
        np.testing.assert_array_equal(eng.maps(k)[0], st["rep_at_temp"])
    eng.close()


def test_split_wolff_sweeps_fp32_equals_unsplit(engine_mod, oracle, monkeypatch):
    """FP32, L = 96 with vacancies and 8 replicas: the split cycle (flag 1024), the unsplit one
    (growth pinned to two CTAs per lattice, which also pins the cycle unsplit), the split cycle
    whose cold slots grow from bond activations decided beforehand, and the unsplit cycle that
    does so for every slot (flag 2048), both cycles with level-free one-CTA growths (flag
    65536), and the split cycle over three, four and five temperature ranges (J1J2C_SPLIT=4,6,
    2,4,6 and 1,2,4,6) give bitwise equal spins, running sums, maps and cluster sizes."""
    jc = engine_mod
    out = []
    base = jc.FLAG_WOLFF | jc.FLAG_GLOBAL
    for i, flags in enumerate((base | jc.FLAG_WOLFF_SPLIT, base | jc.FLAG_WOLFF_CS2,
                               base | jc.FLAG_WOLFF_SPLIT | jc.FLAG_WOLFF_BITS,
                               base | jc.FLAG_WOLFF_BITS,
                               base | jc.FLAG_WOLFF_SPLIT | jc.FLAG_WOLFF_ASYNC,
                               base | jc.FLAG_WOLFF_ASYNC, base | jc.FLAG_WOLFF_SPLIT,
                               base | jc.FLAG_WOLFF_SPLIT, base | jc.FLAG_WOLFF_SPLIT)):
        if i >= 6:
            monkeypatch.setenv("J1J2C_SPLIT", ("4,6", "2,4,6", "1,2,4,6")[i - 6])
        eng, _, _ = _engine(jc, 96, 96, 1, 8, jc.FP32_BATCHED, flags, 0.05)
        eng.run(2, measure=True, restart_swap_phase=True)
        out.append(([eng.spins(0, r) for r in range(8)], eng.slot_sums(0)[0], eng.maps(0)[0],
                    eng.cluster_sizes()))
        eng.close()
    for other in out[1:]:
        for a, b in zip(out[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        for i in (1, 2, 3):
            np.testing.assert_array_equal(out[0][i], other[i])


def test_split_many_ranges_fp32_equals_unsplit(engine_mod, monkeypatch, capfd):
    """FP32, L = 32 lattices in HBM with vacancies, 32 replicas (the count from which the tuner
    also times split lists of three to eight temperature ranges): six ranges pinned by
    J1J2C_SPLIT (one of them 2 slots wide, so its sweeps take two replicas per thread), the
    tuner's choice, and the unsplit cycle give bitwise equal spins, running sums, maps and
    cluster sizes over three cycles; the tuner log shows multi-range candidates timed."""
    jc = engine_mod
    nrep = 32
    base = jc.FLAG_WOLFF | jc.FLAG_GLOBAL
    out = []
    for i, flags in enumerate((base | jc.FLAG_WOLFF_CS2, base | jc.FLAG_WOLFF_SPLIT, base)):
        if i == 1:
            monkeypatch.setenv("J1J2C_SPLIT", "4,12,20,28,30")
        if i == 2:
            monkeypatch.delenv("J1J2C_SPLIT")
            monkeypatch.setenv("J1J2C_TUNE_LOG", "1")
        eng, _, _ = _engine(jc, 32, 32, 1, nrep, jc.FP32_BATCHED, flags, 0.05)
        eng.run(3, measure=True, restart_swap_phase=True)
        out.append(([eng.spins(0, r) for r in range(nrep)], eng.slot_sums(0)[0], eng.maps(0)[0],
                    eng.cluster_sizes()))
        eng.close()
    log = capfd.readouterr().err
    multi = [ln for ln in log.splitlines() if "split L=32" in ln and ln.split(" at ")[1].count(",")]
    assert len(multi) >= 4, log
    for other in out[1:]:
        for a, b in zip(out[0][0], other[0]):
            np.testing.assert_array_equal(a, b)
        for i in (1, 2, 3):
            np.testing.assert_array_equal(out[0][i], other[i])


def _cpu_exact(oracle, L, H, p, betas):
    M = oracle.Model(L, H, p)
    N = L * L * H
    rows = []
    for bits in itertools.product((-1, 1), repeat=N):
        s = np.array(bits[::-1], np.int8)  # any fixed order covers every state
        m, e, sx, sy = M.measurement(s)
        rows.append((e, m, sx, sy, M.nbar(s)))
    a = np.array(rows)
    out = []
    for b in betas:
        Etot = a[:, 0] * N
        w = np.exp(-b * (Etot - Etot.min()))
        Z = w.sum()
        e, m, sx, sy, nb = a.T
        out.append([np.log(Z) - b * Etot.min(), (w * e).sum() / Z, (w * e * e).sum() / Z,
                    (w * abs(m)).sum() / Z, (w * m * m).sum() / Z, (w * m ** 4).sum() / Z,
                    (w * abs(sx)).sum() / Z, (w * sx * sx).sum() / Z, (w * abs(sy)).sum() / Z,
                    (w * sy * sy).sum() / Z, (w * nb).sum() / Z, (w * nb * nb).sum() / Z])
    return np.array(out)


@pytest.mark.parametrize("L,H", [(2, 2), (2, 4)])
def test_enumeration_matches_cpu(engine_mod, oracle, L, H):
    jc = engine_mod
    p = jc.disorder(L, H, 11)
    betas = [0.05, 0.1, 0.125, 0.3]
    gpu = jc.enumerate_exact(L, H, p, betas)
    cpu = _cpu_exact(oracle, L, H, p, betas)
    np.testing.assert_allclose(gpu, cpu, rtol=1e-9, atol=1e-11)


@pytest.mark.parametrize("precision,flags", [(0, 0), (1, 0), (1, 32)])
def test_sampling_matches_exact_4x4x2(engine_mod, oracle, precision, flags):
    """64 independent chains (same disorder, different Philox keys) of a 4-temperature PT ladder
    on 4 x 4 x 2 against the exact averages over all 2^32 states."""
    jc = engine_mod
    L, H, ncopy = 4, 2, 64
    betas = 1.0 / np.array([6.0, 8.0, 10.0, 12.0])
    p = jc.disorder(L, H, SEED)
    exact = jc.enumerate_exact(L, H, p, betas)
    eng, _, _ = _engine(jc, L, H, ncopy, 4, precision, flags, betas=betas, same_disorder=True)
    eng.run(300, measure=False)
    eng.reset_measurements()
    nm = 3000
    eng.run(nm, measure=True)
    sums, cnt = eng.slot_sums(-1)
    assert (cnt == nm).all()
    per = sums.reshape(ncopy, 4, 22) / nm
    checks = {"e": (4, 1), "m2": (2, 4), "abssx": (6, 6), "sx2": (8, 7), "nbar": (16, 10)}
    for name, (si, ei) in checks.items():
        est = per[:, :, si]
        mean, se = est.mean(axis=0), est.std(axis=0, ddof=1) / np.sqrt(ncopy)
        z = np.abs(mean - exact[:, ei]) / np.maximum(se, 1e-12)
        assert (z < 4.5).all(), (name, mean, exact[:, ei], se)
    eng.close()

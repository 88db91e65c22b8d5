"""CPU tests of the oracle: pinned against the committed golden vectors (Ooura-FFT reference build,
Random123 known answers) and against identities of the reference arithmetic."""
import itertools
import json
import math
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers(oracle):
    for kat in json.load(open(os.path.join(GOLDEN, "philox_kat.json"))):
        out = oracle.philox(kat["ctr"], kat["key"])
        assert [int(v) for v in out] == kat["out"]


def test_own_exp_accuracy(oracle):
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(-745, 709, 20000), rng.uniform(-30, 5, 20000),
                         [0.0, -0.0, 1e-300, -1e-300, 1.0, -1.0, 700.0, -700.0, -744.0]])
    for x in xs:
        ref = math.exp(x)
        got = oracle.dexp(float(x))
        if ref == 0.0 or ref < 2.3e-308:
            assert abs(got - ref) <= 5e-324 * 4
        else:
            assert abs(got - ref) <= 1.5 * math.ulp(ref), (x, got, ref)
    assert oracle.dexp(-800.0) == 0.0
    assert math.isinf(oracle.dexp(800.0))


def _golden_corr():
    g = np.load(os.path.join(GOLDEN, "corr3d_golden.npz"))
    cases = {}
    for k in g.files:
        name, part = k.split("__")
        cases.setdefault(name, {})[part] = g[k]
    for name, d in cases.items():
        dims, xi, s, u, m = name.split("_")
        n1, n2, n3 = (int(v) for v in dims[1:].split("x"))
        yield (n1, n2, n3, float(xi[2:]), int(s[1:]), bool(int(u[1:])), float(m[1:])), d


def test_corr3d_restatement_matches_ooura_golden(oracle):
    from oracle import corr3d
    n = 0
    for (n1, n2, n3, xi, seed, uni, mx), d in _golden_corr():
        x = corr3d.make_corr_rand_3d(n1, n2, n3, xi, seed, uni, mx).reshape(-1)
        stride = int(d["stride"][0])
        np.testing.assert_allclose(x[::stride], d["values"], rtol=0, atol=1e-12)
        np.testing.assert_allclose([x.sum(), (x * x).sum()], d["sum"], rtol=1e-12, atol=1e-9)
        n += 1
    assert n >= 5


def test_corr3d_uniform_marginal_and_correlation(oracle):
    from oracle import corr3d
    x = corr3d.make_corr_rand_3d(32, 32, 32, 3.0, 11, True, 2.0)
    assert x.min() >= -2.0 and x.max() <= 2.0
    assert abs(x.mean()) < 0.3
    # uniform on [-2, 2] has variance 4/3 (sample variance is lower because of correlations)
    assert 0.7 < x.var() < 1.45
    g = corr3d.make_corr_rand_3d(32, 32, 32, 3.0, 11, False)
    c1 = np.mean(g * np.roll(g, 1, axis=2)) / np.mean(g * g)
    c4 = np.mean(g * np.roll(g, 4, axis=2)) / np.mean(g * g)
    assert c1 > c4 > 0.0


def test_kiss_uniform_and_seeding(oracle):
    u = oracle.kiss_draw(1, 200000)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.005
    assert not np.array_equal(oracle.kiss_draw(1, 16), oracle.kiss_draw(2, 16))
    np.testing.assert_array_equal(oracle.kiss_draw(7, 16), oracle.kiss_draw(7, 16))
    g = oracle.gkiss_fill(5, 100000)
    assert abs(g.mean()) < 0.02 and abs(g.std() - 1.0) < 0.02


def test_neighbor_table_semantics(oracle):
    L, H = 6, 4
    m = oracle.neighbors(L, H).reshape(10, -1)
    for i in range(L * L * H):
        x, y, z = i % L, (i // L) % L, i // (L * L)

        def site(dx, dy, dz):
            return (x + dx) % L + L * ((y + dy) % L) + L * L * ((z + dz) % H)

        exp = [site(0, 1, 0), site(0, -1, 0), site(1, 0, 0), site(-1, 0, 0), site(1, 1, 0),
               site(-1, 1, 0), site(1, -1, 0), site(-1, -1, 0), site(0, 0, 1), site(0, 0, -1)]
        assert list(m[:, i]) == exp


def _model(oracle, L=6, H=4, seed=3, pp=0.0, bonds=0.0):
    from oracle import corr3d
    p = corr3d.make_corr_rand_3d(L, L, H, 3.0, seed).reshape(-1)
    occu, jh, jv, _ = oracle.setup_vacancies(seed, L, H, pp, bonds, bonds)
    return oracle.Model(L, H, p, occu, jh, jv)


def _bond_energy(M, s):
    """E_total = -sum over bonds of J_eff s_i s_j, bonds counted once (J:2498-2541)."""
    L, H, N = M.L, M.H, M.N
    m = M.m.reshape(10, N)
    occ = M.occu.astype(np.int64)
    ss = s.astype(np.float64) * occ
    J1h, J1v, J2, J3 = M.J
    E = 0.0
    for i in range(N):
        if not occ[i]:
            continue
        j = m[2, i]  # +x bond owned by i
        E -= (J1h * M.jh[i] + M.p[i] + M.p[j]) * ss[i] * ss[j]
        j = m[0, i]  # +y bond owned by i
        E -= (J1v * M.jv[i] - M.p[i] - M.p[j]) * ss[i] * ss[j]
        E -= J2 * ss[i] * (ss[m[4, i]] + ss[m[5, i]])  # (+x,+y) and (-x,+y)
        E -= J3 * ss[i] * ss[m[8, i]]
    return E


@pytest.mark.parametrize("pp,bonds", [(0.0, 0.0), (0.1, 0.0), (0.1, 0.2)])
def test_energy_identity(oracle, pp, bonds):
    M = _model(oracle, pp=pp, bonds=bonds)
    s = oracle.init_spins(9, M.L, M.H, 0)
    obs = M.measurement(s)
    nocc = M.N - M.nimp
    np.testing.assert_allclose(obs[1] * nocc, _bond_energy(M, s), rtol=1e-12, atol=1e-10)
    # the engine's fixed-point energy equals the FP64 sum to ~1e-9 absolute
    ints, acc, o5 = M.replay_measure(s)
    np.testing.assert_allclose(acc * 2.0 ** -33, obs[1] * nocc, rtol=0, atol=1e-6)
    assert o5[0] == obs[0] and o5[2] == obs[2] and o5[3] == obs[3]
    assert o5[4] == M.nbar(s)


def test_metro_sweep_incremental_observables(oracle):
    M = _model(oracle, pp=0.05)
    s = oracle.init_spins(4, M.L, M.H, 0)
    obs = M.measurement(s)
    st = oracle.kiss_state(123)
    for _ in range(20):
        M.metro_sweep(s, 0.11, obs, st)
    np.testing.assert_allclose(obs, M.measurement(s), rtol=0, atol=1e-10)
    M.metro_sweep(s, 0.11, obs, st, rnd=True)
    np.testing.assert_allclose(obs, M.measurement(s), rtol=0, atol=1e-10)


def test_replay_colour_order_is_race_free(oracle):
    """Within a colour no site neighbours another: updating a colour in reversed order gives the
    same configuration as the forward order (checked by replaying with a permuted lattice)."""
    M = _model(oracle, L=8, H=4)
    s = oracle.hot_spins_philox(M.L, M.H, 1, 0, 0)
    m = M.m.reshape(10, M.N)
    col = np.array([(i % 8 & 1) | ((i // 8 % 8) & 1) << 1 | ((i // 64) & 1) << 2
                    for i in range(M.N)])
    assert all((col[m[k]] != col).all() for k in range(10))
    s1 = s.copy()
    f1 = M.replay_sweeps(s1, 0.12, 1, 0, 0, 0, 3)
    s2 = s.copy()
    f2 = M.replay_sweeps(s2, 0.12, 1, 0, 0, 0, 3)
    assert f1 == f2 and np.array_equal(s1, s2) and f1 > 0


def test_replay_pt_bookkeeping(oracle):
    M = _model(oracle, L=8, H=4)
    nrep = 4
    betas = 1.0 / oracle.ladder(nrep, 8.0, 11.5)
    spins = np.stack([oracle.hot_spins_philox(8, 4, 1, 0, r) for r in range(nrep)])
    st = oracle.new_pt_state(spins)
    M.replay_pt(st, betas, 5, 30, 0, 1, 0, True, 1)
    assert sorted(st["rep_at_temp"]) == list(range(nrep))
    assert all(st["temp_of_rep"][st["rep_at_temp"][k]] == k for k in range(nrep))
    assert (st["nmeas"] == 30).all()
    assert st["attempts"][0] == 15 and st["attempts"][1] == 15 and st["attempts"][2] == 15
    assert (st["accepts"][:3] <= st["attempts"][:3]).all()


def test_pt_serial_reference_runs(oracle):
    M = _model(oracle, L=6, H=4)
    betas = 1.0 / oracle.ladder(4, 8.0, 11.5)
    r = M.pt_serial(betas, 5, 20, 40, 1, 1, 0, 0)
    sums = r["sums"]
    assert sums.shape == (4, 22)
    en = sums[:, 4] / 40
    assert (np.diff(en) > -0.5).all()  # energy rises with T (within noise)
    assert (r["attempts"] == 30).all()  # swaps are counted in both loops (J:1224, J:1312)
    assert sorted(r["rep_at_temp"]) == list(range(4))


def test_wolff_restatement_limits(oracle):
    """beta = 0 activates no bond (the cluster is the seed); with ferromagnetic couplings, no
    field and an aligned start, beta -> infinity activates every bond (the whole lattice)."""
    from oracle import corr3d
    L, H = 6, 4
    p = corr3d.make_corr_rand_3d(L, L, H, 3.0, 2).reshape(-1)
    M = oracle.Model(L, H, p)
    s = oracle.init_spins(3, L, H, 0)
    s0 = s.copy()
    assert M.wolff_step(s, 0.0, 1, 0, 0, 7) == 1
    assert int((s != s0).sum()) == 1
    F = oracle.Model(L, H, np.zeros(L * L * H), J1h=1.0, J1v=1.0, J2=1.0, J3=1.0)
    s = np.ones(L * L * H, np.int8)
    assert F.wolff_step(s, 50.0, 1, 0, 0, 7) == L * L * H
    assert (s == -1).all()


def _exact_averages(M, occ, beta):
    """<e>, <|m|>, <m^2> over every spin state of the occupied sites (vacancies 0)."""
    idx = np.flatnonzero(occ)
    rows = []
    for bits in itertools.product((-1, 1), repeat=idx.size):
        s = np.zeros(occ.size, np.int8)
        s[idx] = bits
        m, e, _, _ = M.measurement(s)
        rows.append((e, abs(m), m * m))
    a = np.array(rows)
    E = a[:, 0] * idx.size
    w = np.exp(-beta * (E - E.min()))
    return (a * w[:, None]).sum(0) / w.sum()


@pytest.mark.parametrize("L,H,T,vac,wolff,metro", [(2, 2, 3.0, False, True, False),
                                                   (2, 4, 4.0, False, True, False),
                                                   (2, 4, 4.0, True, True, False),
                                                   (2, 4, 2.5, False, True, True),
                                                   (2, 4, 2.5, True, False, True)])
def test_wolff_restatement_samples_boltzmann(oracle, L, H, T, vac, wolff, metro):
    """The Wolff update as the engine defines it (restated in the oracle) leaves the Boltzmann
    distribution of the reference Hamiltonian invariant: on lattices small enough to enumerate
    every state (L = 2 and H = 2 double the x, y, diagonal and z couplings as in the reference's
    neighbour table), a chain of Wolff updates alone, of the engine's colour-order Metropolis
    sweeps alone, or of both alternating, reproduces the exact <e>, <|m|> and <m^2> within 4.5
    standard errors (batch means over 40 batches).  With a vacancy the vacant site never flips
    and is excluded; diluted J1 bonds carry only the random-field part of their coupling."""
    rng = np.random.default_rng(11)
    N = L * L * H
    p = rng.uniform(-2.0, 2.0, N)
    occ = np.ones(N, np.int8)
    jh = np.ones(N, np.int8)
    jv = np.ones(N, np.int8)
    if vac:  # a vacancy and diluted J1 bonds
        occ[5] = 0
        jh[[1, 9]] = 0
        jv[[4, 14]] = 0
    M = oracle.Model(L, H, p, occ, jh, jv)
    beta = 1.0 / T
    exact = _exact_averages(M, occ, beta)
    s = occ.astype(np.int8).copy()
    nstep, nburn, nb = 120000, 2000, 40
    rec = np.empty((nstep, 3))
    for c in range(nburn + nstep):
        if wolff:
            M.wolff_step(s, beta, 7, 0, 0, c)
        if metro:
            M.replay_sweeps(s, beta, 7, 0, 0, c, 1)
        if c >= nburn:
            m, e, _, _ = M.measurement(s)
            rec[c - nburn] = (e, abs(m), m * m)
    assert (s[occ == 0] == 0).all()
    bm = rec.reshape(nb, -1, 3).mean(1)
    se = bm.std(0, ddof=1) / np.sqrt(nb)
    z = np.abs(bm.mean(0) - exact) / se
    assert (z < 4.5).all(), (bm.mean(0), exact, z)


def test_replay_pt_slot_averages_match_exact(oracle):
    """The engine's PT cycle as the oracle replays it (colour-order Metropolis sweeps, the Philox
    swap on fixed-point lattice energies, observables accumulated by temperature slot) samples
    each slot's Boltzmann distribution: per-slot <e>, <|m|>, <m^2> from the running sums (columns
    en, absmag, mag2) on 2 x 2 x 4 agree with exact enumeration within 4.5 standard errors
    (batch means over 40 chunks of cycles)."""
    L, H, nrep = 2, 4, 4
    N = L * L * H
    rng = np.random.default_rng(13)
    M = oracle.Model(L, H, rng.uniform(-2.0, 2.0, N))
    occ = np.ones(N, np.int8)
    betas = 1.0 / oracle.ladder(nrep, 2.0, 4.0)
    st = oracle.new_pt_state(np.ones((nrep, N), np.int8))
    M.replay_pt(st, betas, 5, 200, 0, 3, 0, False, 1)
    nb, chunk = 40, 600
    cols = [4, 1, 2]
    means = np.empty((nb, nrep, 3))
    for b in range(nb):
        s0, n0 = st["sums"][:, cols].copy(), st["nmeas"].copy()
        M.replay_pt(st, betas, 5, chunk, 200 + b * chunk, 3, 0, True, 1)
        means[b] = (st["sums"][:, cols] - s0) / (st["nmeas"] - n0)[:, None]
    assert st["accepts"][:nrep - 1].min() > 0
    se = means.std(0, ddof=1) / np.sqrt(nb)
    for k in range(nrep):
        exact = _exact_averages(M, occ, betas[k])
        z = np.abs(means[:, k].mean(0) - exact) / se[k]
        assert (z < 4.5).all(), (k, means[:, k].mean(0), exact, z)


@pytest.mark.parametrize("dilute", [False, True])
def test_reference_restatement_samples_exact(oracle, dilute):
    """The oracle's restatement of the reference algorithm itself (one KISS05 stream, sequential
    site order, Metropolis with exp, the PT SERIAL driver and the LOCAL sampler) reproduces the
    exact averages on 2 x 2 x 4, also with a vacancy and diluted J1 bonds: PT per slot over 40
    independent seeds, LOCAL over 40 batches of one long chain, both within 4.5 standard
    errors."""
    L, H, nrep = 2, 4, 4
    N = L * L * H
    rng = np.random.default_rng(17)
    occ = np.ones(N, np.int8)
    jh = np.ones(N, np.int8)
    jv = np.ones(N, np.int8)
    if dilute:
        occ[6] = 0
        jh[[1, 9]] = 0
        jv[[4, 14]] = 0
    M = oracle.Model(L, H, rng.uniform(-2.0, 2.0, N), occ, jh, jv)
    betas = 1.0 / oracle.ladder(nrep, 2.0, 4.0)
    nmess, runs, cols = 400, 40, [4, 1, 2]
    per = np.array([M.pt_serial(betas, 5, 100, nmess, irinit, 1, 0, 0)["sums"][:, cols] / nmess
                    for irinit in range(1, runs + 1)])
    se = per.std(0, ddof=1) / np.sqrt(runs)
    for k in range(nrep):
        z = np.abs(per[:, k].mean(0) - _exact_averages(M, occ, betas[k])) / se[k]
        assert (z < 4.5).all(), (k, z)
    beta = betas[1]
    lists, _ = M.local(occ.copy(), beta, 200, 80000, oracle.kiss_state(5))
    m, e = lists[0], lists[1]
    rec = np.stack([e, np.abs(m), m * m], 1).reshape(40, -1, 3).mean(1)
    z = np.abs(rec.mean(0) - _exact_averages(M, occ, beta)) / (rec.std(0, ddof=1) / np.sqrt(40))
    assert (z < 4.5).all(), z


def test_ladder(oracle):
    t = oracle.ladder(16, 8.0, 11.5)
    np.testing.assert_allclose(t, 8.0 + 3.5 * np.arange(16) / 15, rtol=0, atol=1e-15)
    ts = oracle.ladder(11, 8.0, 11.5, split=True, tmid=9.5, tfrac=0.7)
    assert ts[0] == 8.0 and ts[-1] == 11.5 and ts[7] == 9.5


def test_local_histogram_host_rule_matches_oracle(oracle):
    """The product's LOCAL-histogram rule (Process_data, J:2296-2352) against the oracle's own
    restatement, on random lists, a flat list and a two-value list."""
    import j1j2cuda as jc
    rng = np.random.default_rng(11)
    cases = [rng.normal(-3.8, 0.05, 500), np.full(40, -2.5), np.array([-1.0, -2.0] * 10),
             rng.uniform(-4.0, -3.0, 97)]
    for e in cases:
        for bins in (1, 7, 100):
            c, lo, bs = jc.local_histogram(e, bins)
            c_ref, lo_ref, bs_ref = oracle.local_histogram_ref(e, bins)
            np.testing.assert_array_equal(c, c_ref)
            assert lo == lo_ref and bs == bs_ref


def test_pt_histogram_rule(oracle):
    """J:1514-1523: the first sample fixes the range [e - (|e|+1), e + (|e|+1)] and later
    samples clamp into the end bins."""
    c, lo, bs = oracle.pt_histogram([-2.0, -2.0, -10.0, 5.0, -1.5], 4)
    assert lo == -5.0 and bs == 1.5
    assert c.tolist() == [1.0, 0.0, 3.0, 1.0]

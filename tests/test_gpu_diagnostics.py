"""GPU: measurement diagnostics (per-site local nematic sums, energy histogram, per-cycle trace,
flip counts) against a cycle-by-cycle replay by the oracle, exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 5


def _betas(n, tmin=8.0, tmax=11.5):
    from oracle import oracle as O
    return 1.0 / O.ladder(n, tmin, tmax)


@pytest.mark.parametrize("L,H,pp,slot", [(8, 4, 0.05, 0), (10, 6, 0.0, 2)])
def test_pt_diagnostics_bit_identical(engine_mod, oracle, L, H, pp, slot):
    jc = engine_mod
    nconf, nrep, neq, nmess, bins = 2, 4, 4, 7, 12
    betas = _betas(nrep)
    eng = jc.Engine(L, H, nconf=nconf, nreplica=nrep, precision=jc.FP64_PLAIN, seed=SEED)
    eng.set_diagnostics(locnem_slot=slot, hist_bins=bins, trace_cycles=nmess + 3,
                        flip_counts=True)
    dis = []
    for k in range(nconf):
        p = jc.disorder(L, H, SEED + k)
        occu, _, _, _ = jc.setup_vacancies(SEED + k, L, H, pp)
        eng.set_disorder(k, p, occu)
        eng.set_ladder(k, betas)
        eng.init_spins(k, jc.START_HOT)
        dis.append((p, occu))
    eng.run(neq, measure=False)
    eng.reset_measurements()
    eng.run(nmess, measure=True)
    m = oracle.neighbors(L, H)
    N = L * L * H
    for k in range(nconf):
        p, occu = dis[k]
        M = oracle.Model(L, H, p, occu)
        st = oracle.new_pt_state(np.stack([oracle.hot_spins_philox(L, H, SEED, k, q) * occu
                                           for q in range(nrep)]))
        flips = np.zeros((nrep, N), np.int32)
        M.replay_pt(st, betas, 5, neq, 0, SEED, k, False, 1, flips)
        obs_tr, tor_tr = [], []
        loc_s, loc_n = np.zeros(N, np.int64), np.zeros(N, np.int64)
        for cyc in range(nmess):
            obs = M.replay_pt(st, betas, 5, 1, neq + cyc, SEED, k, True,
                              1 if cyc % 2 == 0 else 2, flips)
            obs_tr.append(obs[st["rep_at_temp"]])
            tor_tr.append(st["temp_of_rep"].copy())
            ds, dn = oracle.locnem_terms(st["spins"][st["rep_at_temp"][slot]], occu, m)
            loc_s += ds
            loc_n += dn
        obs_tr, tor_tr = np.array(obs_tr), np.array(tor_tr)

        gobs, gtor = eng.trace(k)
        np.testing.assert_array_equal(gobs, obs_tr)
        np.testing.assert_array_equal(gtor, tor_tr)

        counts, lo, bs = eng.histogram(k)
        for sl in range(nrep):
            c_ref, lo_ref, bs_ref = oracle.pt_histogram(obs_tr[:, sl, 1], bins)
            np.testing.assert_array_equal(counts[sl], c_ref)
            assert lo[sl] == lo_ref and bs[sl] == bs_ref
        assert counts.sum() == nrep * nmess

        ls, ln, ns = eng.locnem(k)
        assert ns == nmess
        np.testing.assert_array_equal(ls, loc_s.astype(np.float64))
        np.testing.assert_array_equal(ln, loc_n.astype(np.float64))

        fc = eng.flip_counts(k)
        expect = np.where(occu[None, :] == 1, flips, -1)
        np.testing.assert_array_equal(fc, expect)
        assert fc[fc >= 0].sum() > 0
        # the sums and maps are untouched by the diagnostics
        np.testing.assert_array_equal(eng.slot_sums(k)[0], st["sums"])
    eng.close()


def test_flip_counting_leaves_fp32_trajectory_unchanged(engine_mod, oracle):
    """Counting flips switches to the generic kernels; the FP32 trajectory is the same as the
    shape-specialised kernels' (L = 16), and every counted flip is a sign change seen in the
    spins when a single sweep is run."""
    jc = engine_mod
    L, nconf, nrep = 16, 2, 4
    out = []
    for flips in (False, True):
        eng = jc.Engine(L, L, nconf=nconf, nreplica=nrep, precision=jc.FP32_BATCHED, seed=SEED)
        eng.set_diagnostics(flip_counts=flips)
        for k in range(nconf):
            eng.set_disorder(k, jc.disorder(L, L, SEED + k))
            eng.set_ladder(k, _betas(nrep))
            eng.init_spins(k, jc.START_HOT)
        eng.run(6, measure=True)
        out.append(([eng.spins(k, r).copy() for k in range(nconf) for r in range(nrep)],
                    eng.flip_counts(0) if flips else None))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    fc = out[1][1]
    assert fc.min() >= 0 and fc.max() <= 6 * 5 and fc.sum() > 0


def test_diagnostics_errors(engine_mod):
    jc = engine_mod
    eng = jc.Engine(8, 4, nconf=1, nreplica=2, precision=jc.FP64_PLAIN, seed=SEED)
    eng.set_disorder(0, jc.disorder(8, 4, SEED))
    with pytest.raises(jc.J1J2CError):
        eng.locnem(0)  # not enabled
    with pytest.raises(jc.J1J2CError):
        eng.set_diagnostics(hist_bins=-1)
    eng.set_diagnostics(locnem_slot=5)  # beyond this ladder: accumulates nothing
    eng.set_ladder(0, _betas(2))
    eng.init_spins(0, jc.START_HOT)
    eng.run(2, measure=True)
    ls, ln, ns = eng.locnem(0)
    assert ns == 0 and not ls.any() and not ln.any()
    eng.close()


def test_results_files_from_an_engine_run(engine_mod, oracle, tmp_path):
    """A PT run's results written in the reference's formats: the energy column of cfen is the
    disorder average of the slots' mean energies, cfpt holds the engine's swap counts and cfhs
    the engine's histograms divided by NMESS."""
    jc = engine_mod
    L, H, nconf, nrep, nmess, bins = 8, 8, 3, 4, 20, 10
    betas = _betas(nrep)
    eng = jc.Engine(L, H, nconf=nconf, nreplica=nrep, precision=jc.FP32_BATCHED, seed=SEED)
    eng.set_diagnostics(hist_bins=bins, flip_counts=True)
    for k in range(nconf):
        eng.set_disorder(k, jc.disorder(L, H, SEED + k))
        eng.set_ladder(k, betas)
        eng.init_spins(k, jc.START_HOT)
    eng.run(10, measure=False)
    eng.reset_measurements()
    eng.run(nmess, measure=True)
    res = jc.Results(L, H, 1.0 / betas, nconf=nconf, neq=10, nmess=nmess, bins=bins,
                     write_numflips=True)
    for k in range(nconf):
        res.add_engine_conf(eng, k)
    res.write(str(tmp_path))
    en = np.mean([eng.slot_sums(k)[0][:, 4] / nmess for k in range(nconf)], axis=0)
    rows = [ln for ln in open(tmp_path / "cfen00080008.dat").read().splitlines()
            if ln.startswith("   ") and "E" in ln]
    np.testing.assert_allclose([float(r.split()[1]) for r in rows], en, rtol=1e-13)
    pt = open(tmp_path / "cfpt00080008.dat").read().splitlines()
    att = sum(eng.pt_stats(k)[0] for k in range(nconf))
    assert [int(ln.split()[3]) for ln in pt[1:nrep]] == list(att)
    hs = [ln for ln in open(tmp_path / "cfhs00080008.dat").read().splitlines()
          if ln.startswith(" 0.") and len(ln.split()) == 4]
    h = np.mean([eng.histogram(k)[0] for k in range(nconf)], axis=0) / nmess
    np.testing.assert_allclose([float(r.split()[3]) for r in hs], h[:, :bins - 1].reshape(-1),
                               rtol=1e-5, atol=1e-7)
    assert (tmp_path / "cfnu00080008.dat").exists()
    res.close()
    eng.close()

"""GPU: checkpoint / resume.  A run interrupted after some PT cycles, saved, restored into a new
context and continued equals the uninterrupted run bit for bit (spins, maps, counters, running
sums, observables, diagnostics)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 9


def _betas(n):
    from oracle import oracle as O
    return 1.0 / O.ladder(n, 8.0, 11.5)


def _make(jc, groups, precision, flags=0, pp=0.0, diag=None):
    eng = jc.Engine(groups=groups, precision=precision, seed=SEED, flags=flags)
    if diag:
        eng.set_diagnostics(**diag)
    k = 0
    for L, H, n, r in groups:
        for _ in range(n):
            occu = jc.setup_vacancies(SEED + k, L, H, pp)[0] if pp else None
            eng.set_disorder(k, jc.disorder(L, H, SEED + k), occu)
            eng.set_ladder(k, _betas(r))
            eng.init_spins(k, jc.START_HOT)
            k += 1
    return eng


def _snapshot(eng):
    out = []
    for k in range(eng.nconf):
        r = eng.nrep_of(k)
        out.append((np.stack([eng.spins(k, q) for q in range(r)]), eng.maps(k), eng.pt_stats(k),
                    eng.slot_sums(k), eng.observables(k)))
    return out


def _assert_same(a, b):
    for x, y in zip(a, b):
        for u, v in zip(x, y):
            if isinstance(u, tuple):
                for uu, vv in zip(u, v):
                    np.testing.assert_array_equal(np.asarray(uu), np.asarray(vv))
            else:
                np.testing.assert_array_equal(np.asarray(u), np.asarray(v))


CASES = [
    ("fp64", [(8, 4, 2, 4)], 0, 0, 0.05, None),
    ("fp32_mixed", [(16, 16, 2, 4), (8, 8, 3, 3)], 1, 0, 0.0, None),
    ("fp32_wolff_vac", [(12, 12, 2, 3)], 1, 32, 0.05, None),
    ("fp64_diag", [(8, 4, 1, 4)], 0, 0, 0.0,
     dict(locnem_slot=0, hist_bins=10, trace_cycles=20, flip_counts=True)),
]


@pytest.mark.parametrize("name,groups,precision,flags,pp,diag", CASES, ids=[c[0] for c in CASES])
def test_resume_is_bit_identical(engine_mod, name, groups, precision, flags, pp, diag):
    jc = engine_mod
    ref = _make(jc, groups, precision, flags, pp, diag)
    ref.run(3, measure=False)
    ref.reset_measurements()
    ref.run(4, measure=True)
    ref.run(5, measure=True, restart_swap_phase=False)
    want = _snapshot(ref)

    a = _make(jc, groups, precision, flags, pp, diag)
    a.run(3, measure=False)
    a.reset_measurements()
    a.run(4, measure=True)
    blob = a.save_state()
    a.close()

    b = jc.Engine(groups=groups, precision=precision, seed=SEED, flags=flags)
    b.load_state(bytes(blob))
    b.run(5, measure=True, restart_swap_phase=False)
    _assert_same(_snapshot(b), want)
    if diag:
        for k in range(b.nconf):
            np.testing.assert_array_equal(b.flip_counts(k), ref.flip_counts(k))
            np.testing.assert_array_equal(b.histogram(k)[0], ref.histogram(k)[0])
            np.testing.assert_array_equal(b.locnem(k)[1], ref.locnem(k)[1])
            np.testing.assert_array_equal(b.trace(k)[0], ref.trace(k)[0])
    ref.close()
    b.close()


def test_load_rejects_other_parameters(engine_mod):
    jc = engine_mod
    a = _make(jc, [(8, 4, 1, 2)], 0)
    blob = a.save_state()
    a.close()
    for kw in (dict(groups=[(8, 4, 1, 3)], precision=0), dict(groups=[(8, 4, 1, 2)], precision=1),
               dict(groups=[(8, 8, 1, 2)], precision=0)):
        b = jc.Engine(seed=SEED, **kw)
        with pytest.raises(jc.J1J2CError):
            b.load_state(bytes(blob))
        b.close()
    b = jc.Engine(groups=[(8, 4, 1, 2)], precision=0, seed=SEED)
    with pytest.raises(jc.J1J2CError):
        b.load_state(bytes(blob[:100]))
    b.close()

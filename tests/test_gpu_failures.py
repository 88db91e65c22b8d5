"""GPU: failure detection, with every failure made on the host or by a budget that runs out; no
test here faults, traps or hangs the GPU.

* The union-find labelling of the Wolff update gives up after a bounded number of attempts per
  bond; with the budget set to 0 every activated bond gives up, the call reports
  J1J2C_ETIMEOUT, and the context carries on (the error word is cleared once reported).
* A one-shot injected failure of a device allocation (J1J2C_ENOMEM) or of a PT-cycle launch
  (J1J2C_ECUDA), reported without calling CUDA: the failed call changes nothing, the next call
  succeeds, and a failed context creation leaves nothing behind; an autotuner that cannot
  allocate its scratch lattices keeps the untuned form and the run succeeds.

The reference has no recovery of its own: it stops (MPI_ABORT / stop, sim/J1J2_6tv.f90:443-444,
:841-925); these are the engine's own error paths behind the C ABI.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 1


def _engine(jc, L, H, nrep, precision=1, flags=0, betas=None, start=None):
    from oracle import oracle as O
    eng = jc.Engine(L, H, nconf=1, nreplica=nrep, precision=precision, seed=SEED, flags=flags)
    p = jc.disorder(L, H, SEED)
    eng.set_disorder(0, p)
    eng.set_ladder(0, 1.0 / O.ladder(nrep, 8.0, 11.5) if betas is None else betas)
    eng.init_spins(0, jc.START_HOT if start is None else start)
    eng.reset_measurements()
    return eng, p


@pytest.mark.parametrize("flags", [4, 8])  # per-site global labelling; shared-memory slabs
def test_union_find_retry_budget_reports_timeout(engine_mod, flags):
    """A cold ferromagnetic start (T = 1: nearly every satisfied bond is activated), budget 0:
    the per-site form gives up on every activated bond and j1j2c_wolff returns ETIMEOUT (the
    slab form tries each merge once before counting, so it gives up only where a merge was
    contended: ETIMEOUT or success); with the default budget restored the next update and PT
    cycles with Wolff updates succeed, and a cycle under budget 0 fails again with ETIMEOUT."""
    jc = engine_mod
    eng, _ = _engine(jc, 16, 16, 2, flags=flags | jc.FLAG_WOLFF, betas=np.array([1.0, 0.95]),
                     start=jc.START_FER)
    eng.set_retry_budget(0)
    try:
        eng.wolff()
        assert flags == 8, "the per-site form must give up with a budget of 0"
    except jc.J1J2CError as e:
        assert e.code == jc.ETIMEOUT
    eng.set_retry_budget(1 << 20)
    sizes = eng.wolff()
    assert (sizes > 0).all()
    eng.run(3, measure=True)
    s = eng.spins(0, 0)
    assert set(np.unique(s)) <= {-1, 1}
    if flags == 4:
        eng.set_retry_budget(0)
        with pytest.raises(jc.J1J2CError) as e:
            eng.run(1, measure=True)
        assert e.value.code == jc.ETIMEOUT
        eng.set_retry_budget(1 << 20)
        eng.run(2, measure=True)
    with pytest.raises(jc.J1J2CError) as e:
        eng.set_retry_budget(-1)
    assert e.value.code == jc.EINVAL
    eng.close()


def test_injected_allocation_failure(engine_mod):
    """The next device allocation fails: context creation returns ENOMEM (and frees what it had
    allocated); a new context works.  The Wolff labels allocated at first use: j1j2c_wolff
    returns ENOMEM, the next call allocates them and succeeds."""
    jc = engine_mod
    jc.inject_fault(jc.INJECT_ALLOC)
    with pytest.raises(jc.J1J2CError) as e:
        jc.Engine(8, 4, nconf=1, nreplica=2, precision=jc.FP32_BATCHED)
    assert e.value.code == jc.ENOMEM
    eng, _ = _engine(jc, 8, 4, 2, flags=jc.FLAG_GENERIC)
    eng.run(2, measure=True)
    jc.inject_fault(jc.INJECT_ALLOC)
    with pytest.raises(jc.J1J2CError) as e:
        eng.wolff()
    assert e.value.code == jc.ENOMEM
    sizes = eng.wolff()
    assert (sizes > 0).all()
    eng.run(2, measure=True)
    eng.close()
    jc.inject_fault(jc.INJECT_NONE)


def test_tuner_scratch_allocation_failure_falls_back(engine_mod):
    """The next device allocation fails at a Wolff context's first run, where the Wolff tuner
    allocates its scratch lattices: the run goes on with the untuned growth form (one CTA per
    cluster) and gives the same spins and sums as a context that tuned."""
    jc = engine_mod
    out = []
    for inject in (True, False):
        eng, _ = _engine(jc, 12, 10, 8, flags=jc.FLAG_WOLFF)
        if inject:
            jc.inject_fault(jc.INJECT_ALLOC)
        eng.run(3, measure=True, restart_swap_phase=True)
        jc.inject_fault(jc.INJECT_NONE)
        out.append(([eng.spins(0, r) for r in range(8)], eng.slot_sums(0)[0]))
        eng.close()
    for a, b in zip(out[0][0], out[1][0]):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(out[0][1], out[1][1])


def test_injected_launch_failure_changes_nothing(engine_mod, oracle):
    """The next PT-cycle launch fails (ECUDA) before anything is enqueued: after 3 good cycles,
    a failed call and 4 more good cycles, the FP64 state equals the oracle's replay of 7 cycles
    bit for bit; the context is then destroyed normally."""
    jc = engine_mod
    nrep = 4
    eng, p = _engine(jc, 8, 4, nrep, precision=jc.FP64_PLAIN)
    st = oracle.new_pt_state(np.stack([eng.spins(0, r) for r in range(nrep)]))
    betas = 1.0 / oracle.ladder(nrep, 8.0, 11.5)
    eng.run(3, measure=True)
    jc.inject_fault(jc.INJECT_LAUNCH)
    with pytest.raises(jc.J1J2CError) as e:
        eng.run(2, measure=True, restart_swap_phase=False)
    assert e.value.code == jc.ECUDA
    eng.run(4, measure=True, restart_swap_phase=False)
    M = oracle.Model(8, 4, p)
    obs = M.replay_pt(st, betas, 5, 7, 0, SEED, 0, True, 1)
    for r in range(nrep):
        np.testing.assert_array_equal(eng.spins(0, r), st["spins"][r])
    np.testing.assert_array_equal(eng.slot_sums(0)[0], st["sums"])
    np.testing.assert_array_equal(eng.observables(0), obs)
    eng.close()
    with pytest.raises(jc.J1J2CError) as e:
        jc.inject_fault(7)
    assert e.value.code == jc.EINVAL

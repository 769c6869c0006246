"""Sub-islands and ring migration in the oracle (IslandMigration,
proposed model/SG-EMTF.cu:1138-1218, launched at :1409-1410).

The reference splits a block's population into two slots that evolve apart;
every few generations each slot is sorted by fitness (odd-even transposition,
:1114-1136, which keeps equal values in index order) and the i-th best of one
slot replaces the i-th worst of the other when strictly better, both ways at
once from the pre-migration state (:1178-1194).  The oracle generalises the
two slots to a ring of S sub-islands; S = 2 is the reference's exchange.
"""
import numpy as np
import pytest


def _task(orc, NP, D=6, fid=None):
    fid = orc.SPHERE if fid is None else fid
    lo, hi = orc.box(fid)
    return orc.OTask(fid, D, NP, lo, hi, None, None)


@pytest.mark.parametrize("alg", [0, 2])
@pytest.mark.parametrize("S", [2, 4])
def test_trials_draw_within_subisland(orc, alg, S):
    """A member's trial reads only its own sub-island: changing every other
    sub-island leaves it bit-identical."""
    NP, D = 32, 6
    t = _task(orc, NP, D)
    p = orc.params(algorithm=alg, seed=5, subislands=S)
    X = orc.gen_population(5, 0, NP, D, -50.0, 50.0)
    NPs = NP // S
    for s in range(S):
        Y = X.copy()
        other = np.ones(NP, bool)
        other[s * NPs:(s + 1) * NPs] = False
        Y[other] = np.float32(1.25)
        for i in range(s * NPs, (s + 1) * NPs):
            for g in (1, 7):
                assert np.array_equal(orc.trial(p, t, X, g, i), orc.trial(p, t, Y, g, i))


@pytest.mark.parametrize("alg", [0, 2])
def test_one_subisland_is_the_plain_island(orc, alg):
    NP, D = 24, 5
    t = _task(orc, NP, D)
    X = orc.gen_population(3, 0, NP, D, -50.0, 50.0)
    base = orc.params(algorithm=alg, seed=3)
    for S in (0, 1):
        p = orc.params(algorithm=alg, seed=3, subislands=S, mig_interval=2, mig_count=2)
        for i in range(NP):
            assert np.array_equal(orc.trial(p, t, X, 4, i), orc.trial(base, t, X, 4, i))
        assert not any(orc.migration_due(p, g) for g in range(1, 20))


def test_migration_schedule(orc):
    p = orc.params(subislands=2, mig_interval=5)
    assert [g for g in range(1, 22) if orc.migration_due(p, g)] == [6, 11, 16, 21]
    assert not orc.migration_due(orc.params(subislands=2, mig_interval=0), 6)
    assert orc.migration_count(orc.params(subislands=2), 64) == 4
    assert orc.migration_count(orc.params(subislands=4), 16) == 1
    assert orc.migration_count(orc.params(subislands=2, mig_count=3), 64) == 3


def _ring_restatement(X, f, S, m):
    """Plain restatement: rank each sub-island (stable), candidate r of s is
    its r-th best, target the r-th worst of s + 1; strictly better replaces."""
    NP = len(f)
    NPs = NP // S
    order = [s * NPs + np.argsort(f[s * NPs:(s + 1) * NPs], kind="stable") for s in range(S)]
    Y, g = X.copy(), f.copy()
    n = 0
    for s in range(S):
        d = (s + 1) % S
        for r in range(m):
            src, dst = order[s][r], order[d][NPs - 1 - r]
            if f[src] < f[dst]:
                Y[dst], g[dst] = X[src], f[src]
                n += 1
    return Y, g, n


@pytest.mark.parametrize("S,m", [(2, 1), (2, 3), (3, 2), (4, 4)])
def test_migrate_matches_restatement(orc, S, m):
    NP, D = 8 * S, 4
    t = _task(orc, NP, D)
    rng = np.random.default_rng(S * 10 + m)
    # integer genes: sphere values are exact in FP32 and FP64, and repeat,
    # so equal fitness (no replacement) and index-order ties both occur
    X = rng.integers(-3, 4, (NP, D)).astype(np.float32)
    f = np.array([t.eval64(x)[0] for x in X])
    f32 = f.astype(np.float32)
    p = orc.params(subislands=S, mig_interval=1, mig_count=m)
    want_X, want_f, want_n = _ring_restatement(X, f32, S, m)
    for mode in (0, 1):
        Y, g32, g64 = X.copy(), f32.copy(), f.copy()
        n = orc.migrate(p, t, Y, g32, g64, mode)
        assert n == want_n
        assert np.array_equal(Y, want_X)
        assert np.array_equal(g32, want_f)


def test_two_slots_exchange_both_ways(orc):
    """S = 2: slot 0's best improves slot 1's worst and vice versa, decided
    from the pre-migration values (the reference writes both directions from
    one sorted snapshot, SG-EMTF.cu:1178-1194)."""
    NP, D = 8, 2
    t = _task(orc, NP, D)
    X = np.zeros((NP, D), np.float32)
    X[:, 0] = [1, 9, 5, 7, 2, 8, 3, 6]
    f = np.array([t.eval64(x)[0] for x in X])
    p = orc.params(subislands=2, mig_interval=1, mig_count=2)
    Y, f32, f64 = X.copy(), f.astype(np.float32), f.copy()
    assert orc.migrate(p, t, Y, f32, f64, 0) == 4
    # slot 0 = {1, 9, 5, 7}: best 1, 5; slot 1 = {2, 8, 3, 6}: worst 8, 6
    assert list(Y[:, 0]) == [1, 2, 5, 3, 2, 1, 3, 5]

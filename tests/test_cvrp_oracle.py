"""CPU checks of the CVRP oracle: the split decoder against brute force, the
rounded-Euclidean distances, the operators' invariants.  The reference's
CVRP variant is unfinished (proposed model/SG-EMTF_cvrp.cu:731-736 sets every
gene to 1), so these restate the published methods: Prins' split (2004),
order crossover (Davis 1985), swap and 2-opt mutation."""
import itertools

import numpy as np
import pytest


def brute_force(ins, perm):
    n, cap = ins.n, ins.capacity
    D = ins.dist.reshape(n + 1, n + 1)
    d = ins.demand
    best = None
    for mask in range(1 << (n - 1)):
        segs, start = [], 0
        for k in range(n - 1):
            if mask >> k & 1:
                segs.append(perm[start:k + 1])
                start = k + 1
        segs.append(perm[start:])
        if any(d[s].sum() > cap for s in segs):
            continue
        c = sum(int(D[0, s[0]]) + sum(int(D[s[i], s[i + 1]]) for i in range(len(s) - 1)) +
                int(D[s[-1], 0]) for s in segs)
        best = c if best is None else min(best, c)
    return best


def test_split_is_optimal_partition(orc):
    rng = np.random.default_rng(0)
    for _ in range(300):
        n = int(rng.integers(1, 10))
        cap = int(rng.integers(10, 40))
        x, y = rng.integers(0, 1000, n + 1), rng.integers(0, 1000, n + 1)
        d = np.r_[0, rng.integers(1, 11, n)]
        ins = orc.CvrpInstance(0, 0, n, cap, x, y, d)
        perm = (rng.permutation(n) + 1).astype(np.uint8)
        assert ins.split(perm) == brute_force(ins, perm)


def test_split_known_answer(orc):
    # depot at (0,0); customers on a line at x = 3, 6, 9 with demands 2, 2, 2
    x, y, d = [0, 3, 6, 9], [0, 0, 0, 0], [0, 2, 2, 2]
    ins = orc.CvrpInstance(0, 0, 3, 6, x, y, d)
    assert ins.split(np.array([1, 2, 3], np.uint8)) == 18   # one route 0-1-2-3-0
    ins = orc.CvrpInstance(0, 0, 3, 4, x, y, d)
    # capacity 4: {1},{2,3} costs (3+3) + (6+3+9) = 24, {1,2},{3} costs 12 + 18 = 30
    assert ins.split(np.array([1, 2, 3], np.uint8)) == 24


def test_rounded_euclidean(orc):
    ins = orc.CvrpInstance(0, 0, 2, 10, [0, 3, 1], [0, 4, 1], [0, 1, 1])
    D = ins.dist.reshape(3, 3)
    assert D[0, 1] == 5 and D[0, 2] == 1 and D[1, 2] == 4  # sqrt(13) = 3.61 -> 4
    for v in [0, 1, 2, 3, 6, 7, 12, 13, 10**6, 1999998]:
        assert orc.lib().orc_cvrp_round_sqrt(v) == int(np.floor(np.sqrt(v) + 0.5))


def test_seeded_instance_ranges(orc):
    ins = orc.CvrpInstance(7, 3, 100, 50)
    assert ins.x.min() >= 0 and ins.x.max() < 1000 and ins.y.max() < 1000
    assert ins.demand[0] == 0 and ins.demand[1:].min() >= 1 and ins.demand[1:].max() <= 10


def test_children_are_permutations(orc):
    p = orc.cvrp_params(seed=3)
    ins = orc.CvrpInstance(3, 0, 30, 50)
    pop = orc.cvrp_init_population(3, 0, 30, 16)
    for row in pop:
        assert sorted(row) == list(range(1, 31))
    cost = np.array([ins.split(r) for r in pop], np.int32)
    for g in range(1, 6):
        acc = orc.cvrp_generation(p, ins, pop, cost, g)
        for i, row in enumerate(pop):
            assert sorted(row) == list(range(1, 31))
            assert cost[i] == ins.split(row)
    assert acc >= 0


def split_deque(ins, perm):
    """The O(n) deque form of the split (Vidal 2016) that the device runs,
    restated in Python: it must give the label-correcting form's cost."""
    n, W = ins.n, ins.n + 1
    D, q = ins.dist, ins.demand
    dq = []          # (A_i, Q_i), increasing in i and in A
    V = S = Q = 0
    for j in range(1, n + 1):
        c = int(perm[j - 1])
        if j > 1:
            S += int(D[int(perm[j - 2]) * W + c])
        A = V + int(D[c]) - S
        while dq and dq[-1][0] >= A:
            dq.pop()
        dq.append((A, Q))
        Q += int(q[c])
        while Q - dq[0][1] > ins.capacity:
            dq.pop(0)
        V = S + int(D[c]) + dq[0][0]
    return V


@pytest.mark.parametrize("dem_hi", [0, 1, 10, 50])
def test_deque_split_matches_label_correcting(orc, dem_hi):
    rng = np.random.default_rng(dem_hi)
    for _ in range(200):
        n = int(rng.integers(1, 60))
        cap = 50
        x, y = rng.integers(0, 40001, n + 1), rng.integers(0, 40001, n + 1)
        d = np.r_[0, rng.integers(0, dem_hi + 1, n)]
        ins = orc.CvrpInstance(0, 0, n, cap, x, y, d)
        perm = (rng.permutation(n) + 1).astype(np.uint8)
        assert split_deque(ins, perm) == ins.split(perm)


def test_cvrp_migration_oracle(orc):
    """The oracle's CVRP ring migration: S = 1 changes nothing; with groups,
    the r-th cheapest of each group replaces the r-th dearest of the next one
    when strictly cheaper, from the pre-migration state."""
    import numpy as np
    ins = orc.CvrpInstance(4, 0, 12, 20)
    pop = orc.cvrp_init_population(4, 0, 12, 16)
    cost = np.array([ins.split(r) for r in pop], np.int32)
    p1 = orc.cvrp_params(4, subislands=1, mig_interval=1)
    a, ca = pop.copy(), cost.copy()
    assert orc.lib().orc_cvrp_migrate(orc.ctypes.byref(p1), 12, 16, orc._u8(a), orc._i32(ca), 2) == 0
    p = orc.cvrp_params(4, subislands=2, mig_interval=1, mig_count=2)
    b, cb = pop.copy(), cost.copy()
    n = orc.lib().orc_cvrp_migrate(orc.ctypes.byref(p), 12, 16, orc._u8(b), orc._i32(cb), 2)
    want, cw = pop.copy(), cost.copy()
    groups = [list(range(0, 8)), list(range(8, 16))]
    ranked = [sorted(g, key=lambda i: (cost[i], i)) for g in groups]
    moved = 0
    for s in range(2):
        for r in range(2):
            src, dst = ranked[s][r], ranked[(s + 1) % 2][7 - r]
            if cost[src] < cost[dst]:
                want[dst] = pop[src]
                cw[dst] = cost[src]
                moved += 1
    assert n == moved and np.array_equal(b, want) and np.array_equal(cb, cw)
    # not due: generation 1, or off the interval
    p3 = orc.cvrp_params(4, subislands=2, mig_interval=3)
    assert orc.lib().orc_cvrp_migrate(orc.ctypes.byref(p3), 12, 16, orc._u8(pop.copy()),
                                      orc._i32(cost.copy()), 3) == 0

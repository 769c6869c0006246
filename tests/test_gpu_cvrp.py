"""CVRP engine on the GPU against the host replay: instances, initial
islands, generations and elite transfer must match bit for bit (all integer
arithmetic)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def engine(sgemtf, specs, **kw):
    e = sgemtf.CvrpEngine(**kw)
    e.add_instances(specs)
    return e


def check_islands(e, rep):
    for t in range(len(rep.ins)):
        perms, costs = e.population(t)
        np.testing.assert_array_equal(perms, rep.pop[t], err_msg="instance %d" % t)
        np.testing.assert_array_equal(costs, rep.cost[t], err_msg="instance %d" % t)


def test_instances_match_oracle(sgemtf, orc):
    e = engine(sgemtf, [(20, 50), (100, 50), (7, 15)], seed=5)
    for t, (n, cap) in enumerate([(20, 50), (100, 50), (7, 15)]):
        ins = orc.CvrpInstance(5, t, n, cap)
        x, y, d, dist = e.instance(t)
        np.testing.assert_array_equal(x, ins.x)
        np.testing.assert_array_equal(y, ins.y)
        np.testing.assert_array_equal(d, ins.demand)
        np.testing.assert_array_equal(dist, ins.dist)
    e.close()


def test_initial_islands_bit_exact(sgemtf, orc):
    specs = [(20, 50), (100, 50), (1, 10), (57, 30)]
    e = engine(sgemtf, specs, seed=11, pop=64)
    e.reset()
    rep = orc.CvrpReplay(11, [orc.CvrpInstance(11, t, n, c) for t, (n, c) in enumerate(specs)], 64)
    check_islands(e, rep)
    e.close()


@pytest.mark.parametrize("pop", [32, 100, 128])
def test_generations_bit_exact(sgemtf, orc, pop):
    specs = [(20, 50), (100, 50), (37, 25), (64, 80)]
    e = engine(sgemtf, specs, seed=3, pop=pop, p_cross=0.8, p_swap=0.3, p_2opt=0.4)
    rep = orc.CvrpReplay(3, [orc.CvrpInstance(3, t, n, c) for t, (n, c) in enumerate(specs)], pop,
                         p_cross=0.8, p_swap=0.3, p_2opt=0.4)
    for g in (1, 6, 13):
        e.run(g)
        rep.run(g)
        check_islands(e, rep)
    st = e.stats()
    assert st["evaluations"] == len(specs) * pop * (1 + 20)
    e.close()


def related_instances(n, count, rng):
    """Instances on one set of customer sites with different demands: the
    case where a partner's elite tours are useful."""
    x, y = rng.integers(0, 1000, n + 1), rng.integers(0, 1000, n + 1)
    return [(n, 50, x, y, np.r_[0, rng.integers(1, 11, n)]) for _ in range(count)]


def test_transfer_bit_exact(sgemtf, orc):
    rng = np.random.default_rng(0)
    # six related instances of 30 customers, three of 40, two unrelated seeded
    # ones: transfers between equal sizes only
    specs = related_instances(30, 6, rng) + related_instances(40, 3, rng) + [(30, 50), (40, 50)]
    kw = dict(seed=8, pop=64, transfer_interval=5, transfer_rate=0.1)
    e = engine(sgemtf, specs, **kw)
    ins = [orc.CvrpInstance(8, t, *sp) for t, sp in enumerate(specs)]
    rep = orc.CvrpReplay(8, ins, 64, interval=5, rate=0.1)
    for g in (3, 9, 10, 1, 5):
        e.run(g)
        rep.run(g)
        check_islands(e, rep)
    assert e.stats()["transfers_accepted"] == rep.accepted
    assert rep.accepted > 0
    e.close()


def test_explicit_instance_and_best(sgemtf, orc):
    rng = np.random.default_rng(1)
    n = 45
    x, y = rng.integers(0, 40001, n + 1), rng.integers(0, 40001, n + 1)
    d = np.r_[0, rng.integers(0, 20, n)]
    e = engine(sgemtf, [(n, 60, x, y, d), (12, 30)], seed=2, pop=48)
    e.run(25)
    ins = orc.CvrpInstance(2, 0, n, 60, x, y, d)
    perms, costs = e.population(0)
    for r, c in zip(perms, costs):
        assert sorted(r) == list(range(1, n + 1))
        assert ins.split(r) == c
    best = e.best_all()
    assert best[0] == costs.min() and best[1] == e.population(1)[1].min()
    e.close()


def test_best_never_worsens(sgemtf):
    e = engine(sgemtf, [(100, 50)] * 40, seed=4, pop=128, transfer_interval=10)
    e.reset()
    prev = e.best_all()
    for _ in range(4):
        e.run(25)
        cur = e.best_all()
        assert (cur <= prev).all()
        prev = cur
    assert e.stats()["transfers_accepted"] >= 0
    e.close()


def test_argument_errors(sgemtf):
    with pytest.raises(sgemtf.EngineError):
        sgemtf.CvrpEngine(pop=1)
    with pytest.raises(sgemtf.EngineError):
        sgemtf.CvrpEngine(p_cross=1.5)
    e = sgemtf.CvrpEngine(pop=32)
    for bad in ([(0, 10)], [(256, 10)], [(10, 0)],
                [(2, 5, [0, 1, 2], [0, 1, 2], [0, 3, 6])],          # demand above capacity
                [(2, 50, [0, 1, 40001], [0, 1, 2], [0, 3, 6])]):    # coordinate out of range
        with pytest.raises(sgemtf.EngineError):
            e.add_instances(bad)
    e.add_instances([(10, 20)])
    with pytest.raises(sgemtf.EngineError):
        e.population(3)
    with pytest.raises(sgemtf.EngineError):
        e.run(-1)
    e.close()


@pytest.mark.parametrize("case", ["zero_demand", "full_routes", "one_customer", "max_customers",
                                  "far_coords"])
def test_evaluate_edge_instances(sgemtf, orc, case):
    """Device split of random tours against the label-correcting oracle:
    routes as long as the whole tour (zero demands), one customer per route
    (demand = capacity), n = 1, n = 255, coordinates at the 40000 limit."""
    rng = np.random.default_rng(7)
    n, cap, hi_xy = 60, 50, 1000
    if case == "zero_demand":
        d = np.r_[0, np.zeros(n, int)]
    elif case == "full_routes":
        d = np.r_[0, np.full(n, cap)]
    elif case == "one_customer":
        n = 1
        d = np.array([0, 7])
    elif case == "max_customers":
        n = 255
        d = np.r_[0, rng.integers(0, 4, n)]
    else:
        hi_xy = 40000
        d = np.r_[0, rng.integers(1, 11, n)]
    x, y = rng.integers(0, hi_xy + 1, n + 1), rng.integers(0, hi_xy + 1, n + 1)
    e = engine(sgemtf, [(n, cap, x, y, d)], pop=32)
    ins = orc.CvrpInstance(0, 0, n, cap, x, y, d)
    tours = np.stack([rng.permutation(n) + 1 for _ in range(300)]).astype(np.uint8)
    got = e.evaluate(0, tours)
    want = np.array([ins.split(t) for t in tours], np.int32)
    np.testing.assert_array_equal(got, want)
    e.close()


def test_evaluate_rejects_non_permutations(sgemtf):
    e = engine(sgemtf, [(5, 20)], pop=16)
    for bad in ([[1, 2, 3, 4, 4]], [[0, 1, 2, 3, 4]], [[1, 2, 3, 4, 6]]):
        with pytest.raises(sgemtf.EngineError):
            e.evaluate(0, np.array(bad, np.uint8))
    assert len(e.evaluate(0, np.zeros((0, 5), np.uint8))) == 0
    e.close()


def test_long_routes_run_bit_exact(sgemtf, orc):
    """Zero-demand customers make one route hold every customer: the deque
    ring is sized for it and the engine still replays exactly."""
    rng = np.random.default_rng(3)
    n = 90
    x, y = rng.integers(0, 1000, n + 1), rng.integers(0, 1000, n + 1)
    d = np.r_[0, rng.integers(0, 2, n)]
    specs = [(n, 30, x, y, d), (40, 50)]
    e = engine(sgemtf, specs, seed=6, pop=64)
    rep = orc.CvrpReplay(6, [orc.CvrpInstance(6, t, *sp) for t, sp in enumerate(specs)], 64)
    e.run(15)
    rep.run(15)
    check_islands(e, rep)
    e.close()


@pytest.mark.parametrize("cap,dem_hi", [(50, 10), (127, 127), (128, 128), (300, 60),
                                        (32767, 5000), (32768, 9000), (1 << 23, 1 << 20)])
def test_demand_prefix_widths(sgemtf, orc, cap, dem_hi):
    """The deque stores demand prefixes in 1, 2 or 4 bytes depending on the
    largest capacity (2 * capacity must fit): each width, at and past its
    limit, replays the host bit for bit."""
    rng = np.random.default_rng(cap)
    n = 48
    x, y = rng.integers(0, 5000, n + 1), rng.integers(0, 5000, n + 1)
    d = np.r_[0, rng.integers(1, dem_hi + 1, n)]
    specs = [(n, cap, x, y, d), (n, cap, x, y, d[::-1].copy())]
    e = engine(sgemtf, specs, seed=9, pop=32, transfer_interval=4)
    ins = [orc.CvrpInstance(9, t, *sp) for t, sp in enumerate(specs)]
    rep = orc.CvrpReplay(9, ins, 32, interval=4, rate=0.1)
    e.run(10)
    rep.run(10)
    check_islands(e, rep)
    tours = np.stack([rng.permutation(n) + 1 for _ in range(200)]).astype(np.uint8)
    np.testing.assert_array_equal(e.evaluate(0, tours), [ins[0].split(t) for t in tours])
    e.close()


@pytest.mark.parametrize("S,interval,count", [(2, 3, 0), (4, 2, 3)])
def test_subislands_and_migration_bit_exact(sgemtf, orc, S, interval, count):
    """Sub-islands (the reference's IslandMigration, SG-EMTF_cvrp.cu:965-1020):
    tournaments within each group and ring migration between the groups,
    with elite transfer between instances, against the host replay."""
    specs = [(40, 30), (40, 30), (25, 20)]
    ins = [orc.CvrpInstance(12, t, n, c) for t, (n, c) in enumerate(specs)]
    e = engine(sgemtf, specs, seed=12, pop=64, transfer_interval=5, transfer_rate=0.1,
               subislands=S, migration_interval=interval, migration_count=count)
    rep = orc.CvrpReplay(12, ins, 64, interval=5, rate=0.1, subislands=S, mig_interval=interval,
                         mig_count=count)
    e.run(12)
    rep.run(12)
    check_islands(e, rep)
    assert e.stats()["migrations_accepted"] > 0
    e.close()


def test_subisland_arguments(sgemtf):
    for bad in (dict(pop=30, subislands=4), dict(pop=32, subislands=16),
                dict(pop=32, subislands=2, migration_count=9), dict(pop=32, subislands=-1)):
        with pytest.raises(sgemtf.EngineError):
            sgemtf.CvrpEngine(**bad)

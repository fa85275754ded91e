"""Host-side checks of the dispatcher network's oracle and the timing
database (no GPU): the f64 oracle's gradient against central finite
differences, and the database's save / load round trip."""
import numpy as np

from oracle import mlp_ref


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_in, n_h, n_out, n = 5, 7, 3, 11
    cnt = sum(int(np.prod(s)) for _, s in mlp_ref.sizes(n_in, n_h, n_out))
    p = rng.standard_normal(cnt) * 0.5
    x = rng.standard_normal((n, n_in))
    t = rng.standard_normal((n, n_out))
    m = (rng.random((n, n_out)) > 0.3).astype(np.float64)
    loss, g = mlp_ref.loss_and_grad(p, x, t, m, n_in, n_h, n_out)
    h = 1e-6
    fd = np.zeros_like(p)
    for i in range(cnt):
        e = np.zeros_like(p)
        e[i] = h
        fd[i] = (mlp_ref.loss_and_grad(p + e, x, t, m, n_in, n_h, n_out)[0] -
                 mlp_ref.loss_and_grad(p - e, x, t, m, n_in, n_h, n_out)[0]) / (2 * h)
    assert np.allclose(g, fd, rtol=1e-5, atol=1e-8)
    assert loss > 0


def test_oracle_masked_outputs_do_not_contribute():
    rng = np.random.default_rng(1)
    n_in, n_h, n_out, n = 4, 6, 3, 9
    cnt = sum(int(np.prod(s)) for _, s in mlp_ref.sizes(n_in, n_h, n_out))
    p = rng.standard_normal(cnt)
    x = rng.standard_normal((n, n_in))
    t = rng.standard_normal((n, n_out))
    m = np.ones((n, n_out))
    m[:, 1] = 0
    t2 = t.copy()
    t2[:, 1] = 1e6  # garbage where masked
    assert np.allclose(mlp_ref.loss_and_grad(p, x, t, m, n_in, n_h, n_out)[1],
                       mlp_ref.loss_and_grad(p, x, t2, m, n_in, n_h, n_out)[1])


def test_timing_db_round_trip(tmp_path):
    from ndconv.autotune import TimingDB, dispatcher_configs
    specs = dispatcher_configs(50, seed=3)
    db = TimingDB()
    rng = np.random.default_rng(2)
    for s in specs:
        db.add(s, list(rng.random(7)))
    path = str(tmp_path / "t.npz")
    db.save(path)
    db2 = TimingDB.load(path)
    assert [repr(s) for s in db2.specs] == [repr(s) for s in db.specs]
    assert np.allclose(np.array(db2.times), np.array(db.times, np.float32))
    assert db2.lookup(specs[7]) is not None


def test_dispatcher_config_distribution():
    from ndconv.autotune import dispatcher_configs
    specs = dispatcher_configs(3000, seed=1)
    ranks = np.array([s.rank for s in specs])
    assert abs((ranks == 1).mean() - 0.6) < 0.05 and abs((ranks == 2).mean() - 0.35) < 0.05
    two = [s for s in specs if s.rank == 2]
    assert max(max(s.shape) for s in two) <= 4096 and max(max(s.kshape) for s in two) <= 63
    assert all(k % 2 == 1 for s in specs for k in s.kshape)

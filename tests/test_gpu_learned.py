"""Learned point index (workload-5 shape at small sizes): exact pair sets
against the oracle and the LBVH arbiter, GPU training gradients against a CPU
(numpy, FP64) restatement, and what training gains over the untrained model."""
import numpy as np
import pytest

from gpu_util import device_column, device_pairs, pairs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from sedona_gpuspatial import _build, capi, datagen
    import oracle
    _build.build()
    oracle.build(with_ref=False)
    build, boxes, lookups, _ = datagen.workload5(n_build=2_000_000, n_boxes=20_000,
                                                  n_lookups=20_000)
    dev = {name: device_column(capi, col) for name, col in
           (("build", build), ("boxes", boxes), ("lookups", lookups))}
    li = capi.LearnedIndex(leaves=512)
    li.build_device(dev["build"][0])
    return capi, oracle, li, dev, {"build": build, "boxes": boxes, "lookups": lookups}


def _oracle_pairs(oracle, build, probe, pred):
    ob, op = oracle.join(oracle.Geoms(build), oracle.Geoms(probe), pred, nthreads=4)
    return pairs(ob, op)


@pytest.mark.parametrize("probe,pred", [("boxes", "intersects"), ("lookups", "intersects"),
                                        ("boxes", "within"), ("lookups", "equals")])
def test_learned_pairs_match_oracle_and_lbvh_arbiter(env, probe, pred):
    capi, oracle, li, dev, cols = env
    db, dp, n = li.query_device(dev[probe][0], pred)
    got = pairs(*device_pairs(db, dp, n))
    assert n > 200
    assert got == _oracle_pairs(oracle, cols["build"], cols[probe], pred)
    # the LBVH path (the regular join) on the same inputs is the arbiter
    j = capi.SpatialJoin()
    j.build_device(dev["build"][0])
    jb, jp, jn = j.probe_device(dev[probe][0], pred)
    assert got == pairs(*device_pairs(jb, jp, jn))


def test_gpu_gradients_match_cpu_oracle(env):
    capi, oracle, li, dev, cols = env
    m = li.export()
    keys, start, kc = m["keys"].astype(np.float64), m["leaf_start"], m["leaf_kc"]
    rng = np.random.default_rng(3)
    a = m["a"] * (1 + rng.uniform(-0.05, 0.05, li.leaves))
    b = m["b"] + rng.uniform(-20, 20, li.leaves)
    loss, ga, gb = li.loss_and_grad(a, b)
    for l in range(li.leaves):
        s, e = int(start[l]), int(start[l + 1])
        if s == e:
            assert loss[l] == 0 and ga[l] == 0 and gb[l] == 0
            continue
        x = keys[s:e] - float(kc[l])
        r = np.arange(s, e, dtype=np.float64)
        res = a[l] * x + b[l] - r
        np.testing.assert_allclose(loss[l], np.sum(res * res), rtol=1e-9)
        np.testing.assert_allclose(ga[l], np.sum(2 * res * x), rtol=1e-9,
                                   atol=1e-9 * np.sum(np.abs(2 * res * x)))
        np.testing.assert_allclose(gb[l], np.sum(2 * res), rtol=1e-9,
                                   atol=1e-9 * np.sum(np.abs(2 * res)))


def test_trained_model_is_least_squares(env):
    capi, oracle, li, dev, cols = env
    m = li.export()
    loss, ga, gb = li.loss_and_grad(m["a"], m["b"])
    keys, start, kc = m["keys"].astype(np.float64), m["leaf_start"], m["leaf_kc"]
    for l in range(0, li.leaves, 7):
        s, e = int(start[l]), int(start[l + 1])
        if e - s < 2:
            continue
        x = keys[s:e] - float(kc[l])
        if np.ptp(x) == 0:
            continue
        # numpy least squares over the leaf: the GPU Newton step must match
        A = np.stack([x, np.ones_like(x)], 1)
        sol, *_ = np.linalg.lstsq(A, np.arange(s, e, dtype=np.float64), rcond=None)
        np.testing.assert_allclose([m["a"][l], m["b"][l]], sol, rtol=1e-6, atol=1e-6 * (e - s))
        # stationary point: gradient ~ 0 relative to its terms
        assert abs(gb[l]) <= 1e-6 * (e - s) * max(1.0, np.sqrt(loss[l] / (e - s)))


def test_training_gains_over_untrained(env):
    """What the trained model gains: versus its untrained start (the line
    through each leaf's end keys) a lower squared rank error in every leaf
    (least squares), and versus having no model (one binary search over all
    keys, log2(n) steps) far fewer search steps per lookup; the pairs are
    identical either way."""
    capi, oracle, li, dev, cols = env
    results = {}
    for trained in (False, True):
        li.set_trained(trained)
        m = li.export()
        loss, _, _ = li.loss_and_grad(m["a"], m["b"])
        before = li.stats()
        db, dp, n = li.query_device(dev["lookups"][0], "intersects")
        after = li.stats()
        lookups = after["lookups"] - before["lookups"]
        steps = after["search_steps"] - before["search_steps"]
        results[trained] = (pairs(*device_pairs(db, dp, n)), loss, steps / max(1, lookups))
    assert results[True][0] == results[False][0]
    assert np.all(results[True][1] <= results[False][1] * (1 + 1e-9) + 1e-6)
    assert results[True][1].sum() < results[False][1].sum()
    full_search = np.log2(li.stats()["points"])
    assert results[True][2] < 0.75 * full_search


def test_window_fallback_to_lbvh_is_exact(env):
    capi, oracle, li, dev, cols = env
    tiny = capi.LearnedIndex(leaves=64, window=1)  # nearly every leaf over the window
    tiny.build_device(dev["build"][0])
    for probe in ("boxes", "lookups"):
        db, dp, n = tiny.query_device(dev[probe][0], "intersects")
        assert pairs(*device_pairs(db, dp, n)) == _oracle_pairs(oracle, cols["build"],
                                                                cols[probe], "intersects")
    assert tiny.stats()["lbvh_fallbacks"] > 0


def test_window_autotune_keeps_pairs(env):
    """The autotuner picks one of its candidate windows (2^10 .. 2^17, or the
    model's max error) and the pair set does not depend on the window."""
    capi, oracle, li, dev, cols = env
    ref = {p: pairs(*device_pairs(*li.query_device(dev[p][0], "intersects")))
           for p in ("boxes", "lookups")}
    w = li.autotune_window([dev["boxes"][0], dev["lookups"][0]], "intersects")
    st = li.stats()
    assert w in [1 << k for k in range(10, 18)] or w == st["max_err"]
    assert st["window"] == w
    for win in (w, 1, 1 << 20):
        li.set_window(win)
        for p in ("boxes", "lookups"):
            assert pairs(*device_pairs(*li.query_device(dev[p][0], "intersects"))) == ref[p]
    li.set_window(4096)

"""Host-side pieces of the learned preconditioner (no GPU): graph, parameter layout, weights files."""
import numpy as np
import pytest

from smuthi_gb300 import learned


def test_knn_graph_matches_brute_force():
    rng = np.random.default_rng(0)
    xy = rng.uniform(0, 5000, size=(300, 2))
    nbr = learned.knn_graph(xy, 16)
    assert nbr.shape == (300, 17) and nbr.dtype == np.int32
    assert np.array_equal(nbr[:, 0], np.arange(300))
    d2 = ((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    for i in range(0, 300, 7):
        want = np.sort(d2[i])[:16]
        got = np.sort(d2[i, nbr[i, 1:]])
        assert np.allclose(got, want)
        assert i not in nbr[i, 1:]


def test_knn_graph_small_sets():
    xy = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 2.0]])
    nbr = learned.knn_graph(xy, 16)  # k is capped at n - 1
    assert nbr.shape == (3, 3)
    assert list(nbr[0]) == [0, 1, 2]
    assert learned.knn_graph(xy[:1], 4).shape == (1, 1)


@pytest.mark.parametrize("bs", [6, 30, 48])
def test_parameter_layout_and_neumann_start(bs):
    p = learned.init_params(bs, seed=3)
    assert p.dtype == np.float32 and p.size == learned.param_count(bs)
    views = learned.layer_views(p, bs)
    assert len(views) == learned.LAYERS
    for d in views:
        assert d["W1"].shape == (learned.HIDDEN, 4 * bs) and d["W2"].shape == (2 * bs, learned.HIDDEN)
        assert not d["W2"].any() and not d["b2"].any() and list(d["alpha"]) == [1.0, 0.0]
    # views alias the flat vector in order: writing every view covers every parameter exactly once
    q = np.zeros_like(p)
    for li, d in enumerate(learned.layer_views(q, bs)):
        for key in ("W1", "b1", "W2", "b2", "alpha"):
            d[key][...] += 1
    assert np.all(q == 1)
    m = learned.alpha_mask(bs)
    assert m.sum() == 2 * learned.LAYERS


def test_param_count_matches_the_library():
    from smuthi_gb300 import _lib
    try:
        L = _lib.lib()
    except _lib.LibraryMissing:
        pytest.skip("library not built")
    for bs in (6, 30, 48, 64):
        assert L.sg_precond_param_count(bs) == learned.param_count(bs)
    assert L.sg_precond_param_count(65) == -1


@pytest.mark.parametrize("name", ["precond_c5", "precond_c2"])
def test_shipped_weights_load(name):
    p = learned.load_params(name, 30)
    assert np.all(np.isfinite(p))
    with pytest.raises(ValueError):
        learned.load_params(name, 48)
    d = np.load(learned.DATA_DIR + "/" + name + ".npz")
    assert "report" in d.files  # the selection report travels with the weights

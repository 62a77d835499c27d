"""The learned router: its hand-written training kernels against an FP64 CPU
restatement, training that reduces the loss, and routed queries that stay
exact while searching fewer lists."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bf16_round(a):
    """Round float32 to the nearest BF16 value (ties to even), as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def unpack(p, d, H, L):
    sizes = [H * d, H, H * H, H, L * H, L]
    out, o = [], 0
    for s in sizes:
        out.append(p[o:o + s])
        o += s
    W1, b1, W2, b2, W3, b3 = out
    return W1.reshape(H, d), b1, W2.reshape(H, H), b2, W3.reshape(L, H), b3


def cpu_loss_and_grads(p, X, y, d, H, L, t=None):
    """FP64 forward/backward of the router (weights rounded to BF16 as the GPU
    uses them); t: the distance head's targets (NaN for none), whose row is the
    last of W3 and b3."""
    from scipy.special import erf
    T = 0 if t is None else 1
    W1, b1, W2, b2, W3, b3 = unpack(p.astype(np.float64), d, H, L + T)
    W1, W2, W3 = bf16_round(W1), bf16_round(W2), bf16_round(W3)
    X = X.astype(np.float64)
    B = X.shape[0]
    gelu = lambda x: 0.5 * x * (1 + erf(x / np.sqrt(2)))
    dgelu = lambda x: 0.5 * (1 + erf(x / np.sqrt(2))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)
    h1 = X @ W1.T + b1
    a1 = gelu(h1)
    h2 = a1 @ W2.T + b2
    a2 = gelu(h2)
    zall = a2 @ W3.T + b3
    z = zall[:, :L]
    zmax = z.max(1, keepdims=True)
    lse = zmax[:, 0] + np.log(np.exp(z - zmax).sum(1))
    per = lse - z[np.arange(B), y]
    dz = np.exp(z - lse[:, None])
    dz[np.arange(B), y] -= 1
    if T:
        ok = np.isfinite(t)
        e = np.where(ok, zall[:, L] - np.where(ok, t, 0.0), 0.0)
        per = per + e * e
        dz = np.concatenate([dz, (2 * e)[:, None]], 1)
    loss = per.mean()
    dz /= B
    gW3 = dz.T @ a2
    gb3 = dz.sum(0)
    da2 = dz @ W3 * dgelu(h2)
    gW2 = da2.T @ a1
    gb2 = da2.sum(0)
    da1 = da2 @ W2 * dgelu(h1)
    gW1 = da1.T @ X
    gb1 = da1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])


@pytest.mark.parametrize("d,H,L,B", [(16, 32, 40, 24), (128, 64, 300, 70)])
def test_router_gradients_match_cpu(rbc, d, H, L, B):
    rng = np.random.default_rng(d + L)
    r = rbc.Router(d, H, L, seed=3)
    p = (rng.standard_normal(r.num_params()) * 0.3).astype(np.float32)
    r.set_params(p)
    X = rng.standard_normal((B, d)).astype(np.float32)
    y = rng.integers(0, L, B).astype(np.int32)
    loss, g = r.gradients(X, y)
    rl, rg = cpu_loss_and_grads(p, X, y, d, H, L)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    scale = np.abs(rg).max()
    np.testing.assert_allclose(g, rg, rtol=2e-3, atol=2e-4 * scale)
    np.testing.assert_array_equal(r.get_params(), p)  # gradients alone do not update
    r.close()


def test_router_training_reduces_loss(rbc, oracle):
    # labels = the mixture component of each row: learnable from the row alone.
    # With sigma = 0 the generator returns each row's component mean, so the
    # distinct noise-free rows enumerate the components.
    import torch
    d, L = 32, 64
    X = rbc.synth(1, 5, 0, 20000, d, ncomp=L, sigma_lo=0.03, sigma_hi=0.03)
    Xz = oracle.synth(1, 5, 0, 20000, d, ncomp=L, sigma_lo=0.0, sigma_hi=0.0)
    _, labels = np.unique(Xz, axis=0, return_inverse=True)
    labels = torch.from_numpy(labels.astype(np.int32).ravel())
    r = rbc.Router(d, 128, int(labels.max().item()) + 1, seed=1)
    first, _ = r.gradients(X[:1024], labels[:1024])
    last = r.train(X, labels, epochs=8, batch=512, lr=3e-3, seed=2)
    assert last < 0.25 * first, (first, last)
    pred = r.logits(X[:4000]).argmax(1).cpu()
    assert (pred == labels[:4000].long()).float().mean().item() > 0.9
    r.close()


def test_routed_queries_are_exact_and_probe_fewer_lists(rbc, oracle):
    import torch
    n, d, nr, ncomp = 120000, 64, 512, 400
    X = rbc.synth(1, 11, 0, n, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qtr = rbc.synth(1, 11, 2, 40000, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qte = rbc.synth(1, 11, 1, 1500, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    idx = rbc.Index(X, nr, seed=4, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    labels = idx.owner_labels(Qtr)
    r = rbc.Router(d, 256, nr, seed=7)
    r.train(Qtr, labels, epochs=6, batch=1024, lr=2e-3, seed=3)
    test_labels = idx.owner_labels(Qte).cpu()
    top1 = r.logits(Qte).argmax(1).cpu()
    router_recall = (top1 == test_labels.long()).float().mean().item()
    ids0, d0 = idx.query(Qte, 10)
    plain = idx.stats()
    idx.set_router(r, probes=2)
    ids1, d1 = idx.query(Qte, 10, mode=rbc.QUERY_ROUTED)
    routed = idx.stats()
    assert (ids0 == ids1).all() and (d0 == d1).all()  # routing never changes the exact answer
    ri, rd = oracle.knn(X.cpu().numpy(), Qte[:300].cpu().numpy(), 10)
    np.testing.assert_array_equal(rbc.u32(ids1[:300]), ri)
    for mode in (rbc.QUERY_EXACT_TC, rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED):  # learned + BF16 form
        ids2, d2 = idx.query(Qte, 10, mode=mode)
        assert (ids2 == ids0).all() and (d2 == d0).all()
    tc_routed = idx.stats()
    # the router's picks alone in the tensor form's probe round (no nearest
    # list): still exact, the nearest representative's distance feeds the bound
    idx.set_tc_tuning(rbc.TC_ROUTER_ONLY, 2048)
    ids3, d3 = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED)
    assert (ids3 == ids0).all() and (d3 == d0).all()
    ids4, d4 = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC)  # unrouted: one nearest list
    assert (ids4 == ids0).all() and (d4 == d0).all()
    print(f"router top-1 recall {router_recall:.3f}; lists/query plain {plain['lists_probed'] / 1500:.2f} "
          f"routed {routed['lists_probed'] / 1500:.2f}; pairs/query plain {plain['point_pairs'] / 1500:.0f} "
          f"routed {routed['point_pairs'] / 1500:.0f}; tensor routed pairs/query {tc_routed['point_pairs'] / 1500:.0f}"
          f" fallbacks {tc_routed['fallback_queries']}")
    assert router_recall > 0.5
    assert routed["point_pairs"] < plain["point_pairs"]
    idx.close()
    r.close()


def test_tensor_core_inference_matches_training_forward(rbc):
    """The routed queries' tensor-core inference (BF16 activations) against an
    FP64 restatement of the training forward: same argmax nearly everywhere,
    logits within BF16 rounding of the activations."""
    from scipy.special import erf
    rng = np.random.default_rng(5)
    d, H, L, B = 72, 128, 300, 700
    r = rbc.Router(d, H, L, seed=9)
    p = r.get_params()
    X = rng.standard_normal((B, d)).astype(np.float32)
    z = r.logits(X).cpu().numpy().astype(np.float64)
    W1, b1, W2, b2, W3, b3 = unpack(p.astype(np.float64), d, H, L)
    W1, W2, W3 = bf16_round(W1), bf16_round(W2), bf16_round(W3)
    gelu = lambda x: 0.5 * x * (1 + erf(x / np.sqrt(2)))
    a1 = bf16_round(gelu(bf16_round(X) @ W1.T + b1))
    a2 = bf16_round(gelu(a1 @ W2.T + b2))
    ref = a2 @ W3.T + b3
    scale = np.abs(ref).max()
    assert np.abs(z - ref).max() <= 2e-2 * scale
    assert (z.argmax(1) == ref.argmax(1)).mean() > 0.97
    r.close()


def test_router_only_probes_gain_over_the_nearest_list(rbc, oracle):
    """The tensor form on one index, one probed list per query either way: the
    nearest representative's list (unrouted) or the router's top pick
    (RBC_TC_ROUTER_ONLY).  Both are exact; the router's list holds the
    nearest neighbour more often, so its probe round leaves a tighter k-th
    distance and the pruning round searches fewer (query, row) pairs."""
    n, d, nr, ncomp = 200000, 64, 1024, 600
    X = rbc.synth(1, 13, 0, n, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qtr = rbc.synth(1, 13, 2, 60000, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qte = rbc.synth(1, 13, 1, 2000, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    idx = rbc.Index(X, nr, seed=5, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    r = rbc.Router(d, 256, nr, seed=8)
    r.train(Qtr, idx.owner_labels(Qtr), epochs=6, batch=1024, lr=2e-3, seed=4)
    idx.set_router(r, probes=1)
    idx.set_tc_tuning(1, 1 << 20)
    ids0, d0 = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC)
    nearest = idx.stats()
    idx.set_tc_tuning(rbc.TC_ROUTER_ONLY, 1 << 20)
    ids1, d1 = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED)
    routed = idx.stats()
    ri, rd = oracle.knn(X.cpu().numpy(), Qte.cpu().numpy(), 10)
    np.testing.assert_array_equal(rbc.u32(ids0), ri)
    np.testing.assert_array_equal(rbc.u32(ids1), ri)
    assert (d0 == d1).all()
    print(f"one probed list: nearest {nearest['point_pairs'] / 2000:.0f} pairs, {nearest['lists_probed'] / 2000:.1f}"
          f" lists per query; router {routed['point_pairs'] / 2000:.0f} pairs, "
          f"{routed['lists_probed'] / 2000:.1f} lists per query")
    # the gain: the router's probe leaves the pruning fewer pairs and lists
    assert routed["point_pairs"] < nearest["point_pairs"], (routed, nearest)
    assert routed["lists_probed"] <= nearest["lists_probed"], (routed, nearest)
    idx.close()
    r.close()


@pytest.mark.parametrize("d,H,L,B", [(16, 32, 40, 24), (128, 64, 300, 70)])
def test_distance_head_gradients_match_cpu(rbc, d, H, L, B):
    """Both heads' loss and every gradient against the FP64 restatement; rows
    without a target (NaN) train the list head only."""
    rng = np.random.default_rng(d + L + 1)
    r = rbc.Router(d, H, L, seed=3, distance_head=True)
    assert r.num_params() == H * d + H + H * H + H + (L + 1) * H + L + 1
    p = (rng.standard_normal(r.num_params()) * 0.3).astype(np.float32)
    r.set_params(p)
    X = rng.standard_normal((B, d)).astype(np.float32)
    y = rng.integers(0, L, B).astype(np.int32)
    t = rng.standard_normal(B).astype(np.float32)
    t[::5] = np.nan
    loss, g = r.gradients_with_distance(X, y, t)
    rl, rg = cpu_loss_and_grads(p, X, y, d, H, L, t.astype(np.float64))
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    scale = np.abs(rg).max()
    np.testing.assert_allclose(g, rg, rtol=2e-3, atol=2e-4 * scale)
    r.close()


def test_predicted_distance_plan_is_exact(rbc, oracle):
    """A router whose distance head predicts each query's 10th-neighbour
    distance, attached with probes = 0: the tensor form skips its probe round
    and plans with the prediction.  Answers equal the oracle's; with the
    calibrated margin few queries are answered twice, and with a margin far
    too small most are -- and every answer is still exact."""
    n, d, nr, ncomp = 120000, 64, 512, 400
    X = rbc.synth(1, 17, 0, n, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qtr = rbc.synth(1, 17, 2, 50000, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    Qte = rbc.synth(1, 17, 1, 1500, d, ncomp=ncomp, sigma_lo=0.02, sigma_hi=0.1)
    idx = rbc.Index(X, nr, seed=4, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    labels, dist, near = idx.router_labels(Qtr, 10)
    r = rbc.Router(d, 256, nr, seed=7, distance_head=True)
    r.train_with_distance(Qtr, labels, dist, near, epochs=6, batch=1024, lr=2e-3, seed=3)
    mu, sigma, margin = r.distance_params()
    _, true_d, te_near = idx.router_labels(Qte, 10)
    pred = r.predict_distance(Qte, te_near)
    ratio = (pred / true_d).cpu().numpy()
    # the calibrated margin puts nearly every prediction above the true distance
    assert np.isfinite(ratio).all() and np.median(ratio) > 1.0 and (ratio < 1).mean() < 0.03, (np.median(ratio), margin)
    ri, rd = oracle.knn(X.cpu().numpy(), Qte.cpu().numpy(), 10)
    idx.set_router(r, probes=0)
    ids, dists = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED)
    np.testing.assert_array_equal(rbc.u32(ids), ri)
    np.testing.assert_array_equal(dists.cpu().numpy(), rd)
    calibrated = idx.stats()["fallback_queries"]
    assert calibrated <= 1500 // 10, calibrated
    r.set_distance_margin(margin - 3.0)  # predictions far below the true distances
    ids, dists = idx.query(Qte, 10, mode=rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED)
    np.testing.assert_array_equal(rbc.u32(ids), ri)
    np.testing.assert_array_equal(dists.cpu().numpy(), rd)
    again = idx.stats()["fallback_queries"]
    assert again > 1500 // 2 and len(idx.fallback_queries()) == again, again
    print(f"distance head: median predicted / true {np.median(ratio):.3f}, margin {margin:.3f} (x sigma {sigma:.3f});"
          f" answered twice: {calibrated} calibrated, {again} with the margin lowered by 3")
    with pytest.raises(rbc.RBCError):
        idx.set_router(rbc.Router(d, 64, nr, seed=1), probes=0)  # no distance head
    idx.close()
    r.close()


@pytest.mark.parametrize("d,H,L,P", [(128, 512, 4096, 2), (64, 256, 1000, 5), (32, 128, 300, 16)])
def test_fused_top_lists_match_the_logits(rbc, d, H, L, P):
    """The routed queries' probe picks come from the last layer fused with the
    selection (no logits in memory); they equal the top P of the logits the
    unfused tensor-core GEMMs write, ties to the lower list, wherever the
    gap to the next logit is clear of rounding."""
    rng = np.random.default_rng(L + P)
    r = rbc.Router(d, H, L, seed=11)
    X = rng.standard_normal((3000, d)).astype(np.float32)
    top = rbc.u32(r.top_lists(X, P)).astype(np.int64)
    z = r.logits(X).cpu().numpy().astype(np.float64)
    order = np.argsort(-z, axis=1, kind="stable")[:, :P + 1]
    zs = np.take_along_axis(z, order, 1)
    gap = np.abs(np.diff(zs, axis=1)).min(1) > 1e-4 * np.abs(zs).max(1)
    assert gap.mean() > 0.9
    np.testing.assert_array_equal(top[gap], order[gap, :P])
    assert (top >= 0).all() and (top < L).all()
    r.close()


def test_autotune_may_skip_an_unhelpful_router(rbc, oracle):
    """An untrained router (random weights) on i.i.d. integer features: its
    picks are noise.  rbc_autotune_tc in routed mode also times the nearest
    lists without the router; whichever it keeps, routed tensor-form answers
    stay the oracle's, and when it skips the router (info()["tc_unrouted"])
    a routed call does exactly the unrouted call's work.  Setting the knobs
    by hand or attaching the router again consults the router again."""
    n, d, nr = 60000, 64, 128
    X = rbc.synth(2, 17, 0, n, d)
    Q = rbc.synth(2, 17, 1, 400, d)
    Qt = rbc.synth(2, 17, 3, 2000, d)
    idx = rbc.Index(X, nr, seed=3, flags=rbc.BUILD_PARTITION | rbc.BUILD_BF16)
    r = rbc.Router(d, 64, nr, seed=9)
    idx.set_router(r, probes=2)
    routed = rbc.QUERY_EXACT_TC | rbc.QUERY_ROUTED
    idx.autotune_tc(Qt, 10, routed)
    skip = idx.info()["tc_unrouted"]
    assert skip in (0, 1)
    ri, rd = oracle.knn(X.cpu().numpy(), Q.cpu().numpy(), 10)
    ids, dists = idx.query(Q, 10, mode=routed)
    np.testing.assert_array_equal(rbc.u32(ids), ri)
    np.testing.assert_array_equal(dists.cpu().numpy(), rd)
    st_routed = idx.stats()
    if skip:
        idx.query(Q, 10, mode=rbc.QUERY_EXACT_TC)
        st_plain = idx.stats()
        assert st_routed["lists_probed"] == st_plain["lists_probed"]
        assert st_routed["point_pairs"] == st_plain["point_pairs"]
    p, rows = idx.tc_tuning()
    idx.set_tc_tuning(p if p else 2, rows)
    assert idx.info()["tc_unrouted"] == 0
    idx.set_router(r, probes=2)
    assert idx.info()["tc_unrouted"] == 0
    ids, dists = idx.query(Q, 10, mode=routed)
    np.testing.assert_array_equal(rbc.u32(ids), ri)
    idx.close()
    r.close()

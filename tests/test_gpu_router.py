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


def cpu_loss_and_grads(p, X, y, d, H, L):
    """FP64 forward/backward of the router (weights rounded to BF16 as the GPU uses them)."""
    from scipy.special import erf
    W1, b1, W2, b2, W3, b3 = unpack(p.astype(np.float64), d, H, L)
    W1, W2, W3 = bf16_round(W1), bf16_round(W2), bf16_round(W3)
    X = X.astype(np.float64)
    B = X.shape[0]
    gelu = lambda x: 0.5 * x * (1 + erf(x / np.sqrt(2)))
    dgelu = lambda x: 0.5 * (1 + erf(x / np.sqrt(2))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)
    h1 = X @ W1.T + b1
    a1 = gelu(h1)
    h2 = a1 @ W2.T + b2
    a2 = gelu(h2)
    z = a2 @ W3.T + b3
    zmax = z.max(1, keepdims=True)
    lse = zmax[:, 0] + np.log(np.exp(z - zmax).sum(1))
    loss = (lse - z[np.arange(B), y]).mean()
    dz = np.exp(z - lse[:, None])
    dz[np.arange(B), y] -= 1
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

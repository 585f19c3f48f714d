"""The learned GK15 depth proposal: its device kernels against the CPU oracle, its training, and what it gains.

- features, inference logits and the training loss/gradient of the tensor-core kernels agree with the oracle's
  double-precision restatement of the same network (BF16 rounding at the same places);
- training on the plain integrator's depth labels lowers the loss;
- ablation: on held-out pairs the proposal evaluates fewer panels than the plain integrator, and its result is
  bit-identical wherever the proposed depth does not exceed the plain tree's shallowest leaf, and within the
  integration tolerance's order everywhere.
"""

import numpy as np
import pytest

from antipodal_gb300 import synth

pytestmark = pytest.mark.gpu

SLICES = {"W1": (0, 1024), "b1": (1024, 1088), "W2": (1088, 5184), "b2": (5184, 5248), "W3": (5248, 6272),
          "b3": (6272, 6288)}


def patch_pairs(seed, n_patches, n_queries):
    curves, q, x0 = synth.bezier_patches(seed=seed, n_patches=n_patches, n_queries=n_queries)
    return curves, q, x0


@pytest.fixture(scope="module")
def trained(gwn):
    """A network trained on seeded patches (seed 21), shared by the tests that need one."""
    disp = gwn.CudaDispatcher(device=0)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    net = gwn.LearnedGK15Proposal(disp, seed=3, n_classes=11, alpha=0.02)
    curves, q, x0 = patch_pairs(21, 64, 600)
    hist = net.fit(q, x0, curves, cfg, steps=800, batch=4096, lr=2e-3, seed=5)
    yield disp, net, cfg, hist
    net.close()
    disp.close()


def test_features_match_oracle(gwn, disp, oracle):
    curves, q, x0 = patch_pairs(31, 8, 200)
    net = gwn.LearnedGK15Proposal(disp, seed=1)
    got = net.features(q, x0, curves, 1e-10)
    ref = oracle.param_features(q, x0, curves, 1e-10)
    assert got.shape == ref.shape == (len(q) * len(curves), 12)
    assert np.isfinite(got).all()
    d = np.abs(got - ref)
    # float vs double evaluation of the same formulas; a nearest-segment tie may pick another segment
    assert (d > 1e-3).mean() < 1e-3, d.max(axis=0)
    assert np.median(d) < 1e-6


def test_inference_logits_match_oracle(gwn, disp, oracle):
    curves, q, x0 = patch_pairs(32, 4, 100)
    net = gwn.LearnedGK15Proposal(disp, seed=7)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    logits = np.empty((len(q) * len(curves), 16), np.float32)
    net.start_depths(disp, q, x0, curves, cfg, logits=logits)
    feats = net.features(q, x0, curves, cfg.tol)
    ref = oracle.mlp_logits(net.params, feats)
    d = np.abs(logits - ref)
    scale = np.abs(ref).max()
    assert np.quantile(d, 0.99) < 1e-3 * scale + 1e-4, (np.quantile(d, 0.99), scale)
    assert d.max() < 5e-2 * scale


@pytest.mark.parametrize("n", [128, 1000, 4096])
def test_loss_and_gradient_match_oracle(gwn, disp, oracle, n):
    curves, q, x0 = patch_pairs(33, 16, max(1, n // 64))
    net = gwn.LearnedGK15Proposal(disp, seed=11)
    feats = net.features(q, x0, curves, 1e-10)[:n]
    rng = np.random.default_rng(n)
    labels = rng.integers(0, 11, size=len(feats)).astype(np.uint8)
    loss, g = net.loss_grad(feats, labels)
    rloss, rg = oracle.mlp_loss_grad(net.params, feats, labels, 11)
    assert abs(loss - rloss) <= 1e-4 * abs(rloss)
    for name, (a, b) in SLICES.items():
        gd, rd = g[a:b].astype(np.float64), rg[a:b]
        scale = np.abs(rd).max()
        assert scale > 0, name
        rel = np.linalg.norm(gd - rd) / np.linalg.norm(rd)
        assert rel < 1e-2, (name, rel)
        assert np.abs(gd - rd).max() < 3e-2 * scale, (name, np.abs(gd - rd).max(), scale)
    # the padded input columns of W1 get no gradient
    w1 = g[0:1024].reshape(64, 16)
    assert (w1[:, 12:] == 0).all()


def test_training_lowers_the_loss(trained):
    _, _, _, hist = trained
    assert np.isfinite(hist).all()
    assert hist[-100:].mean() < 0.75 * hist[:20].mean(), (hist[:20].mean(), hist[-100:].mean())


def test_ablation_proposal_saves_panels_at_equal_accuracy(gwn, trained):
    disp, net, cfg, _ = trained
    curves, q, x0 = patch_pairs(22, 48, 400)  # held out: other patches, other queries
    n, c = len(q), len(curves)
    st = np.empty((n, c), np.uint32)
    nodes_plain = np.empty(n, np.int32)
    plain = np.empty(n)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, plain, x0, curves, cfg, pair_stats=st,
                                              nodes_per_query=nodes_plain)
    _, dmin, _ = gwn.unpack_pair_stats(st)
    start = net.start_depths(disp, q, x0, curves, cfg)
    nodes = np.empty(n, np.int32)
    got = np.empty(n)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, got, x0, curves, cfg, integrator=net, nodes_per_query=nodes)
    # same call with the explicit start depths gives the same bits
    again = np.empty(n)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, again, x0, curves, cfg, start_depth=start)
    assert np.array_equal(again, got)
    over = start.astype(int) > dmin
    saved = 1.0 - nodes.sum() / nodes_plain.sum()
    print(f"panels saved {saved:.3f}, overshooting pairs {over.mean():.4f}")
    # the best any start-depth proposal can do is the labels themselves
    best = np.empty(n, np.int32)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, np.empty(n), x0, curves, cfg, start_depth=dmin.astype(np.uint8),
                                              nodes_per_query=best)
    best_saved = 1.0 - best.sum() / nodes_plain.sum()
    print(f"panels saved {saved:.3f} (labels as proposal: {best_saved:.3f}), overshooting pairs {over.mean():.4f}")
    assert over.mean() < 0.05
    assert saved > 0.08 and saved > 0.35 * best_saved
    exact_rows = ~over.any(axis=1)
    assert np.array_equal(got[exact_rows], plain[exact_rows])
    # elsewhere both trees are partitions of [0, 1] whose accepted error estimates sum to <= tol per curve
    assert np.abs(got - plain).max() <= 2 * cfg.tol * c / (4 * np.pi)
    # a larger alpha starts deeper (the labels are the shallowest accepted depth, a lower bound on the cheapest start:
    # most of a pair's tree lies deeper): fewer panels still, and still within the plain bound
    deep = gwn.LearnedGK15Proposal(disp, n_classes=11, alpha=0.9, params=net.params)
    nodes_deep = np.empty(n, np.int32)
    got_deep = np.empty(n)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, got_deep, x0, curves, cfg, integrator=deep,
                                              nodes_per_query=nodes_deep)
    print(f"panels saved at alpha 0.9: {1.0 - nodes_deep.sum() / nodes_plain.sum():.3f}")
    assert nodes_deep.sum() < nodes.sum()
    assert np.abs(got_deep - plain).max() <= 2 * cfg.tol * c / (4 * np.pi)
    deep.close()
    # without the network (all start depths 0) the plain integrator is reproduced exactly
    zero = np.zeros((n, c), np.uint8)
    base = np.empty(n)
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, base, x0, curves, cfg, start_depth=zero)
    assert np.array_equal(base, plain)


def test_alpha_is_monotone_and_save_load_roundtrip(gwn, trained, tmp_path):
    disp, net, cfg, _ = trained
    curves, q, x0 = patch_pairs(23, 8, 100)
    lo = gwn.LearnedGK15Proposal(disp, n_classes=11, alpha=0.005, params=net.params)
    hi = gwn.LearnedGK15Proposal(disp, n_classes=11, alpha=0.3, params=net.params)
    s_lo = lo.start_depths(disp, q, x0, curves, cfg)
    s_hi = hi.start_depths(disp, q, x0, curves, cfg)
    assert (s_hi >= s_lo).all()
    assert (s_hi <= cfg.max_depth).all()
    path = tmp_path / "proposal.npz"
    net.save(path)
    back = gwn.LearnedGK15Proposal.load(disp, path)
    assert np.array_equal(back.params, net.params)
    assert np.array_equal(back.start_depths(disp, q, x0, curves, cfg), net.start_depths(disp, q, x0, curves, cfg))
    # min_depth raises every proposal; max_depth caps it
    deep = gwn.IntegrateConfig(3, 4, cfg.tol)
    s = net.start_depths(disp, q, x0, curves, deep)
    assert (s >= 3).all() and (s <= 4).all()
    lo.close(), hi.close(), back.close()


def test_device_tensor_inputs(gwn, trained):
    torch = pytest.importorskip("torch")
    disp, net, cfg, _ = trained
    curves, q, x0 = patch_pairs(24, 4, 64)
    host = net.start_depths(disp, q, x0, curves, cfg)
    qd, cd = torch.from_numpy(q).cuda(), torch.from_numpy(curves).cuda()
    dev = net.start_depths(disp, qd, x0, cd, cfg)
    torch.cuda.synchronize()
    assert dev.is_cuda and np.array_equal(dev.cpu().numpy(), host)
    lab = net.labels(qd, x0, cd, cfg)
    assert lab.is_cuda and lab.numel() == len(q) * len(curves)


def test_errors(gwn, disp):
    net = gwn.LearnedGK15Proposal(disp, seed=1)
    with pytest.raises(ValueError):
        net.params = np.zeros(5, np.float32)
    bad = net.params
    bad[7] = np.nan
    with pytest.raises(gwn.GwnError):
        net.params = bad
    f = np.zeros((256, 12), np.float32)
    lab = np.zeros(256, np.uint8)
    with pytest.raises(gwn.GwnError):
        net.train(f, lab, steps=1, batch=100)  # not a multiple of 128
    net.n_classes = 17
    with pytest.raises(gwn.GwnError):
        net.loss_grad(f, lab)


def test_panel_log_counts_the_plain_tree(gwn, disp):
    """Every split panel of the plain tree is logged once: split entries = sum over pairs of (leaves - 1)."""
    curves, q, x0 = patch_pairs(41, 8, 200)
    cfg = gwn.IntegrateConfig(0, 10, 1e-10)
    st = np.empty((len(q), len(curves)), np.uint32)
    out = np.empty(len(q))
    gwn.eval_gwnr_parametric_batch_fractional(disp, q, out, x0, curves, cfg, pair_stats=st)
    lv, _, dmax = gwn.unpack_pair_stats(st)
    net = gwn.LearnedGK15Proposal(disp, seed=2)
    feats, labels = net.panel_data(q, x0, curves, cfg, capacity=2_000_000)
    assert np.isfinite(feats).all()
    assert int((labels == 0).sum()) == int((lv - 1).sum())
    # accepted entries: the leaves above max_depth (forced leaves at max_depth are not logged)
    assert int(labels.sum()) <= int(lv.sum())
    net.close()


def test_panel_network_skips_panels_at_equal_accuracy(gwn, trained):
    disp, net, cfg, _ = trained
    tc, tq, tx = patch_pairs(21, 64, 300)
    disp.set_param_precision("mixed")
    try:
        hist = net.fit_panels(tq, tx, tc, cfg, beta=0.02, capacity=3_000_000, steps=800, batch=8192, lr=2e-3)
        assert hist[-100:].mean() < 0.8 * hist[:20].mean()
        curves, q, x0 = patch_pairs(22, 48, 300)  # held out
        n = len(q)
        base, nb = np.empty(n), np.empty(n, np.int32)
        gwn.eval_gwnr_parametric_batch_fractional(disp, q, base, x0, curves, cfg, nodes_per_query=nb)
        got, ng = np.empty(n), np.empty(n, np.int32)
        gwn.eval_gwnr_parametric_batch_fractional(disp, q, got, x0, curves, cfg, integrator=net, nodes_per_query=ng)
        panel, start_only = net.panel, None
        net.panel = None
        try:
            start_only = np.empty(n, np.int32)
            gwn.eval_gwnr_parametric_batch_fractional(disp, q, np.empty(n), x0, curves, cfg, integrator=net,
                                                      nodes_per_query=start_only)
        finally:
            net.panel = panel
        print(f"panels: plain {nb.sum()}, start depth only {start_only.sum()}, start depth + panel net {ng.sum()}")
        assert ng.sum() < start_only.sum() < nb.sum()
        assert np.abs(got - base).max() <= 1e-8
    finally:
        disp.set_param_precision("exact")


def test_panel_network_save_load(gwn, trained, tmp_path):
    disp, net, cfg, _ = trained
    if net.panel is None:
        pytest.skip("the panel network is trained by the previous test")
    path = tmp_path / "p.npz"
    net.save(path)
    back = gwn.LearnedGK15Proposal.load(disp, path)
    assert back.panel is not None and np.array_equal(back.panel.params, net.panel.params)
    assert back.panel.alpha == net.panel.alpha
    back.close()

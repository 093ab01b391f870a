"""The learned BC1 path (ntg_compress_chain_learned): the pruned ordering search and its full-fit
fallback are exact where they claim to be, and a trained network gains over the same search
without it while staying within 0.5% of the plain cluster fit's RMSE."""
import numpy as np
import pytest

import ntg
from ntg import learned

pytestmark = pytest.mark.gpu

INF = float("inf")


def _same(a, b):
    return (a.view(-1, 8) == b.view(-1, 8)).all(dim=1).float().mean().item()


@pytest.fixture(scope="module")
def net():
    n = ntg.MLP(seed=21)
    yield n
    n.close()


@pytest.mark.parametrize("kind,size", [(0, 96), (1, 128), (1, 37)])
def test_wide_radius_is_the_full_search(ctx, net, kind, size):
    """Radius 16 covers every ordering: the pruned search is the full search, block for block."""
    import torch
    img = learned.generator_texture(kind, size, 40 + size)
    opt = learned.generator_options(kind)
    d = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=16, margin=INF)
    assert _same(out, plain) == 1.0
    assert st["full_fit"] == 0


def test_true_orderings_at_radius_zero(ctx):
    """The targets' orderings, fed back as proposals, pick exactly the full fit's blocks."""
    import torch
    size = 128
    img = learned.generator_texture(1, size, 77)
    opt = learned.generator_options(1)
    d = torch.from_numpy(img).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    t = ctx.chain_targets(d, size, size, opt, plain)
    y = torch.zeros((t.shape[0], 16), dtype=torch.float32, device="cuda")
    y[:, :6] = t[:, :6]
    out, _ = ctx.compress_chain_proposed(y, d, size, size, opt, radius=0, margin=INF)
    assert _same(out, plain) == 1.0


def test_descent_from_true_orderings_stays(ctx):
    """A steepest descent started at the full search's own orderings finds nothing strictly better one
    step away (the start is the global minimum), so it keeps them: the full fit's blocks."""
    import torch
    size = 128
    img = learned.generator_texture(2, size, 79)
    opt = learned.generator_options(2)
    d = torch.from_numpy(img).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    t = ctx.chain_targets(d, size, size, opt, plain)
    y = torch.zeros((t.shape[0], 16), dtype=torch.float32, device="cuda")
    y[:, :6] = t[:, :6]
    out, st = ctx.compress_chain_proposed(y, d, size, size, opt, radius=ntg.NTG_PROPOSAL_DESCENT | 4, margin=INF)
    assert _same(out, plain) == 1.0
    assert st["full_fit"] == 0


def test_fallback_list_is_the_full_fit(ctx, net):
    """A margin of -1 sends every fitted block to the full fit through the device-side list."""
    import torch
    size = 96
    img = learned.generator_texture(0, size, 5)
    opt = learned.generator_options(0)
    d = torch.from_numpy(img).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=0, margin=-1.0)
    assert _same(out, plain) == 1.0
    assert st["full_fit"] > 0


def test_features_and_targets(ctx):
    import torch
    size = 64
    img = learned.generator_texture(1, size, 3)
    opt = learned.generator_options(1)
    d = torch.from_numpy(img).cuda()
    x = ctx.chain_features(d, size, size, opt)
    t = ctx.chain_targets(d, size, size, opt, ctx.compress_chain(d, size, size, opt))
    n = sum(ntg.nblocks(w, h) for w, h in ntg.chain_levels(size, size))
    assert x.shape == (n, 48) and t.shape == (n, 8)
    assert float(x.min()) >= 0.0 and float(x.max()) <= 1.0
    f = t[:, :5]
    assert float(f.min()) >= 0.0 and float(f.max()) <= 1.0 + 1e-6
    assert bool((t[:, 0] <= t[:, 1] + 1e-6).all()) and bool((t[:, 1] <= t[:, 2] + 1e-6).all())


def test_trained_network_gains_over_no_network(ctx):
    """Trained on chains of the two generators, evaluated on a separate seed: the learned pruned
    search stays within 0.5% of the plain fit's RMSE and finds the full fit's exact block more
    often than the same search seeded without the network."""
    import torch
    x, t = learned.training_set(ctx, 1 << 20, seed=0x7E57, size=1024)
    net = ntg.MLP(seed=9)
    try:
        losses = learned.train(net, x, t, steps=1024, batch=8192, lr=2e-3)
        assert losses[-64:].mean() < 0.5 * losses[:8].mean()
        size = 512
        img = learned.generator_texture(1, size, 0xE7A1)
        opt = learned.generator_options(1)
        d = torch.from_numpy(img).cuda()
        plain = ctx.compress_chain(d, size, size, opt)
        rp = learned.chain_rmse(ctx, d, size, size, opt, plain)
        out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=2, margin=INF)
        rl = learned.chain_rmse(ctx, d, size, size, opt, out)
        assert rl <= 1.005 * rp, (rl, rp)
        base, _ = ctx.compress_chain_proposed(learned.uniform_proposals(plain.numel() // 8), d, size, size, opt,
                                              radius=2, margin=INF)
        assert _same(out, plain) > _same(base, plain) + 0.05, (_same(out, plain), _same(base, plain))
        assert st["orderings"] < 200 * (st["kept"] + st["full_fit"])  # versus up to 1120 per block in full
    finally:
        net.close()


# ---- BC3 colour: squish Compress4 splits proposed by the network ----

def _same16(a, b):
    return (a.view(-1, 16) == b.view(-1, 16)).all(dim=1).float().mean().item()


@pytest.mark.parametrize("kind,size", [(3, 96), (4, 128), (3, 37)])
def test_bc3_wide_radius_is_the_full_search(ctx, net, kind, size):
    """Radius 16 covers every split of up to 16 colours: the pruned search is the full squish search."""
    import torch
    img = learned.generator_texture(kind, size, 50 + size)
    opt = learned.generator_options(kind)
    d = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=16, margin=INF)
    assert _same16(out, plain) == 1.0
    assert st["full_fit"] == 0


@pytest.mark.parametrize("kind", [3, 4])
def test_bc3_true_splits_at_radius_zero(ctx, kind):
    """The targets' splits, fed back as proposals, pick exactly the full fit's blocks."""
    import torch
    size = 128
    img = learned.generator_texture(kind, size, 78)
    opt = learned.generator_options(kind)
    d = torch.from_numpy(img).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    t = ctx.chain_targets(d, size, size, opt, plain)
    y = torch.zeros((t.shape[0], 16), dtype=torch.float32, device="cuda")
    y[:, :6] = t[:, :6]
    out, st = ctx.compress_chain_proposed(y, d, size, size, opt, radius=0, margin=INF)
    assert _same16(out, plain) == 1.0
    assert st["orderings"] <= st["kept"]  # at most one split per fitted block


def test_bc3_fallback_list_is_the_full_fit(ctx, net):
    """A margin of -1 sends every fitted block to the full k_bc3 through the device-side list."""
    import torch
    size = 96
    img = learned.generator_texture(3, size, 6)
    opt = learned.generator_options(3)
    d = torch.from_numpy(img).cuda()
    plain = ctx.compress_chain(d, size, size, opt)
    out, st = ctx.compress_chain_learned(net, d, size, size, opt, radius=0, margin=-1.0)
    assert _same16(out, plain) == 1.0
    assert st["full_fit"] > 0


def test_bc3_features_and_targets(ctx):
    import torch
    size = 64
    img = learned.generator_texture(4, size, 3)
    opt = learned.generator_options(4)
    d = torch.from_numpy(img).cuda()
    x = ctx.chain_features(d, size, size, opt)
    t = ctx.chain_targets(d, size, size, opt, ctx.compress_chain(d, size, size, opt))
    n = sum(ntg.nblocks(w, h) for w, h in ntg.chain_levels(size, size))
    assert x.shape == (n, 48) and t.shape == (n, 8)
    assert float(x.min()) >= 0.0 and float(x.max()) <= 1.0
    f = t[:, :3]
    assert float(f.min()) >= 0.0 and float(f.max()) <= 1.0 + 1e-6
    assert bool((t[:, 0] <= t[:, 1] + 1e-6).all()) and bool((t[:, 1] <= t[:, 2] + 1e-6).all())
    assert bool(torch.isfinite(t[:, 5]).all())


def test_batch_bc3_proposal_wide_radius_is_exact(ctx, net, tmp_path, monkeypatch):
    """A batch with proposals for both BC1 and BC3 at a radius that covers every ordering and split
    gives the plain batch's bytes; clearing them restores the plain graph."""
    import torch
    import ntg.synth as synth
    monkeypatch.setenv("NTG_TUNE_CACHE", str(tmp_path / "tune.json"))
    textures, refs = [], []
    for i, (w, h, fmt) in enumerate([(128, 64, 4), (64, 64, 1), (96, 96, 4), (32, 32, 7), (200, 40, 4)]):
        img = synth.batch_texture(w, h, fmt, 300 + i)
        opt = ntg.ChainOptions.make(format=fmt, quality=1, filter=ntg.FILTER_KAISER,
                                    alpha_mode=ntg.ALPHA_TRANSPARENCY if fmt == 4 else ntg.ALPHA_NONE)
        d_in = torch.from_numpy(img.reshape(-1).view(np.uint32)).cuda()
        refs.append(ctx.compress_chain(d_in, w, h, opt).clone())
        textures.append((d_in, w, h, opt, torch.zeros_like(refs[-1])))
    b = ntg.Batch(ctx, textures)
    net3 = ntg.MLP(seed=23)
    try:
        launches = b.info()["launches"]
        b.set_proposal(net, radius=16, margin=INF)
        b.set_proposal(net3, radius=16, margin=INF, format=ntg.FORMAT_BC3)
        assert b.info()["launches"] == launches + 6
        for t in textures:
            t[4].zero_()
        b.launch()
        torch.cuda.synchronize()
        for t, r in zip(textures, refs):
            assert torch.equal(t[4], r)
        st = b.proposal_stats(format=ntg.FORMAT_BC3)
        assert st["kept"] > 0 and st["full_fit"] == 0
        b.set_proposal(None, format=ntg.FORMAT_BC3)
        b.set_proposal(None)
        assert b.info()["launches"] == launches
    finally:
        b.close()
        net3.close()

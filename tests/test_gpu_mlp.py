"""Learned gas optics on the GPU: the hand-written training kernels against
the CPU restatement (oracle/mlp_oracle.py), the inference kernel against the
training forward pass, training on plain-taumol layers, and the per-layer
fallback to taumol."""
import numpy as np
import pytest

import mlp_oracle as M
from brams_gb300 import rrtmg_lw as R
from brams_gb300 import surrogate as S
from brams_gb300.profiles import ProfileSpec, make_state

pytestmark = pytest.mark.gpu


def _torch():
    import torch

    return torch


def _rand_batch(rows, seed):
    rs = np.random.default_rng(seed)
    x = np.zeros((rows, 16), dtype=np.float32)
    x[:, :9] = rs.normal(size=(rows, 9))
    x = M.bf16(x)
    t = np.zeros((rows, 288), dtype=np.float32)
    t[:, :280] = rs.normal(size=(rows, 280))
    return x, t


def _dev_bf16(x):
    torch = _torch()
    return torch.from_numpy(x).cuda().to(torch.bfloat16)


def test_gradients_match_cpu_oracle(ctx):
    torch = _torch()
    mlp = R.Mlp(ctx, seed=11)
    p, _ = mlp.params()
    rows = 256
    x, t = _rand_batch(rows, 5)
    grad = torch.zeros(R.MLP_NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    mlp.gradients(rows, _dev_bf16(x), torch.from_numpy(t).cuda(), grad, loss)
    torch.cuda.synchronize()
    g_gpu = grad.cpu().numpy().astype(np.float64)
    l_ref, g_ref = M.forward_backward(p, x, t, emulate=True)
    assert abs(loss.item() - l_ref) <= 1e-4 * l_ref
    G, Gr = M.unpack(g_gpu), M.unpack(g_ref)
    for k in G:
        scale = np.abs(Gr[k]).max()
        err = np.abs(G[k] - Gr[k]).max()
        assert err <= 2e-2 * scale + 1e-12, (k, err, scale)
    # and against the float64 network without bf16 rounding (looser)
    _, g64 = M.forward_backward(p, x.astype(np.float64), t.astype(np.float64), emulate=False)
    assert np.abs(g_gpu - g64).max() <= 0.1 * np.abs(g64).max()


def test_forward_outputs_match_cpu(ctx):
    torch = _torch()
    mlp = R.Mlp(ctx, seed=12)
    p, _ = mlp.params()
    rows = 64
    x, t = _rand_batch(rows, 6)
    y = torch.zeros((rows, 288), dtype=torch.float32, device="cuda")
    mlp.forward(rows, _dev_bf16(x), y)
    P = M.unpack(p)
    a = x.astype(np.float32)
    for l in (1, 2, 3):
        a = M.bf16(M.silu(a @ M.bf16(P[f"W{l}"].astype(np.float32)) + P[f"b{l}"].astype(np.float32)))
    ref = a @ M.bf16(P["W4"].astype(np.float32)) + P["b4"].astype(np.float32)
    got = y.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-2 * (np.abs(ref).max() + 1.0)


@pytest.fixture(scope="module")
def trained(ctx):
    """A network trained briefly on plain-taumol layers (small set)."""
    mlp, info = S.train(ctx, n_layers=120_000, epochs=6, batch=4096, lr=3e-3, seed=3, log=lambda *a: None)
    return mlp, info


def test_training_reduces_loss(trained):
    _, info = trained
    h = info["loss"]
    assert h[-1] < 0.5 * h[0], h
    assert np.isfinite(h).all()


def test_inference_kernel_matches_training_forward(ctx, trained):
    torch = _torch()
    mlp, _ = trained
    spec = ProfileSpec(ncol=40, nlay=45, seed=77, t_noise=4.0, h2o_sigma=0.5)
    g = S.DeviceGrid(make_state(spec))
    rows = 40 * 45
    tau = torch.zeros((rows, 140), dtype=torch.float16, device="cuda")
    frac = torch.zeros((rows, 140), dtype=torch.float16, device="cuda")
    flag = torch.zeros(rows, dtype=torch.uint8, device="cuda")
    mlp.infer(g.desc(), tau, frac, flag)
    # same layers through the training path
    feat = torch.zeros((rows, 9), dtype=torch.float32, device="cuda")
    t0 = torch.zeros((rows, 140), dtype=torch.float32, device="cuda")
    f0 = torch.zeros((rows, 140), dtype=torch.float32, device="cuda")
    mlp.samples(g.desc(icld=0), feat, t0, f0)
    x = torch.zeros((rows, 16), dtype=torch.bfloat16, device="cuda")
    mlp.prepare(rows, feat, t0, f0, x, None)
    y = torch.zeros((rows, 288), dtype=torch.float32, device="cuda")
    mlp.forward(rows, x, y)
    _, norm = mlp.params()
    mu, sd = norm[50:338], norm[338:626]
    yv = y.cpu().numpy() * sd + mu
    ok = flag.cpu().numpy() == 1
    assert ok.mean() > 0.9
    got_tau, got_frac = tau.float().cpu().numpy(), frac.float().cpu().numpy()
    # the outputs are stored as binary16: relative steps of 2^-11 down to
    # 2^-14, absolute steps of 2^-24 below it (optical depths under 6e-5)
    want = np.minimum(np.exp(yv[ok, :140]), 65504.0)
    tol = 1e-3 * (np.abs(yv[:, :140]).max() + 1)
    normal = want >= 2.0**-14
    assert np.abs(np.log(got_tau[ok][normal]) - yv[ok, :140][normal]).max() <= tol + 2.0**-10
    assert np.abs(got_tau[ok][~normal] - want[~normal]).max() <= 2.0**-23 + tol * 2.0**-14
    assert np.abs(got_frac[ok] - yv[ok, 140:280]).max() <= 1e-3 + 2.0**-11


def test_out_of_range_layers_fall_back_to_taumol(ctx, trained):
    """A column whose every layer lies outside the training range must give
    exactly the plain solver's result; in-range columns use the network."""
    torch = _torch()
    mlp, _ = trained
    spec = ProfileSpec(ncol=24, nlay=45, seed=78, t_noise=4.0, h2o_sigma=0.5)
    st = make_state(spec)
    st["tlay"][:3] += 200.0  # every layer far outside the training temperatures
    st["tlev"][:3] += 200.0
    import pyoracle

    tauc = pyoracle.cldprop_columns(st)
    g1, g2 = S.DeviceGrid(st, tauc), S.DeviceGrid(st, tauc)
    ctx.rrtmg_lw_batch_device([g1.desc(seed0=5)])
    mlp.batch([g2.desc(seed0=5)])
    torch.cuda.synchronize()
    a, b = g1.outputs(), g2.outputs()
    for k in a:
        assert np.array_equal(a[k][:3], b[k][:3]), k
    assert not np.array_equal(a["uflx"][3:], b["uflx"][3:])
    assert ctx.sync_status() == 0


def test_tcgen05_inference_matches_mma_sync(ctx, trained):
    """The tensor-memory (tcgen05) inference kernel against the warp-MMA one on
    the same layers: same flags, outputs equal up to the order of the fp32
    sums (which can move a bf16 activation by one unit in the last place)."""
    torch = _torch()
    mlp, _ = trained
    spec = ProfileSpec(ncol=203, nlay=45, seed=79, t_noise=4.0, h2o_sigma=0.5)  # 9135 rows: a partial last tile
    g = S.DeviceGrid(make_state(spec))
    rows = 203 * 45
    out = {}
    for eng in (R.MLP_MMA_SYNC, R.MLP_TCGEN05):
        mlp.set_engine(eng)
        tau = torch.full((rows, 140), -1.0, dtype=torch.float16, device="cuda")
        frac = torch.full((rows, 140), -1.0, dtype=torch.float16, device="cuda")
        flag = torch.full((rows,), 7, dtype=torch.uint8, device="cuda")
        mlp.infer(g.desc(), tau, frac, flag)
        torch.cuda.synchronize()
        out[eng] = (tau.float().cpu().numpy(), frac.float().cpu().numpy(), flag.cpu().numpy())
    mlp.set_engine(R.MLP_MMA_SYNC)
    assert ctx.sync_status() == 0
    (t0, f0, g0), (t1, f1, g1) = out[R.MLP_MMA_SYNC], out[R.MLP_TCGEN05]
    assert np.array_equal(g0, g1)
    assert (t1 >= 0).all() and np.isfinite(t1).all()
    normal = (t0 >= 2.0**-14) & (t1 >= 2.0**-14)  # binary16 normal range
    assert np.abs(np.log(t1[normal]) - np.log(t0[normal])).max() <= 0.05
    assert np.abs(np.log(t1[normal]) - np.log(t0[normal])).mean() <= 2e-3
    assert np.abs(t1[~normal] - t0[~normal]).max() <= 0.05 * 2.0**-14
    assert np.abs(f1 - f0).max() <= 5e-3


def test_what_the_network_gains(ctx):
    """The trained network (brams_gb300/data/lw_mlp.gbmlp) against the method
    without it on 32,768 columns x 45 layers: the column kernel with learned
    gas optics must beat the one running taumol by at least 1.3x at a
    heating-rate RMSE within 0.1 K/day of the FP64 oracle; the inference cost
    and the end-to-end ratio are printed (run with -s)."""
    import pyoracle

    torch = _torch()
    ncol, nlay = 32768, 45
    spec = ProfileSpec(ncol=ncol, nlay=nlay, seed=80, t_noise=4.0, h2o_sigma=0.5)
    st = make_state(spec)
    tauc = pyoracle.cldprop_columns(st)
    mlp = S.load(ctx)
    gp, gl = S.DeviceGrid(st, tauc), S.DeviceGrid(st, tauc)
    rows = ncol * nlay
    tau = torch.empty((rows, 140), dtype=torch.float16, device="cuda")
    frac = torch.empty_like(tau)
    flag = torch.empty(rows, dtype=torch.uint8, device="cuda")

    def timeit(fn, n=5):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(n):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    t_plain = timeit(lambda: ctx.rrtmg_lw_batch_device([gp.desc(seed0=9)]))
    t_inf = timeit(lambda: mlp.infer(gl.desc(seed0=9), tau, frac, flag))
    lg = gl.desc(seed0=9, sur_tau=tau, sur_frac=frac, sur_flag=flag)
    t_col = timeit(lambda: ctx.rrtmg_lw_batch_device([lg]))
    assert ctx.sync_status() == 0
    n = 1024
    sub = {k: np.asfortranarray(v[:n]) for k, v in st.items()}
    mc = pyoracle.mcica_per_column(sub, np.asfortranarray(tauc[:, :n]), icld=3, base_seed=9)
    ref = pyoracle.rrtmg_lw(sub, mc, icld=3)
    hr_l = gl.outputs()["hr"][:n]
    rmse = float(np.sqrt(np.mean((hr_l - ref["hr"]) ** 2)))
    print(f"\nplain column kernel {t_plain:.2f} ms; learned: inference {t_inf:.2f} ms + column kernel {t_col:.2f} ms "
          f"(column kernel {t_plain / t_col:.2f}x, end to end {t_plain / (t_inf + t_col):.2f}x); "
          f"heating-rate RMSE {rmse:.4f} K/day, layers on the network {flag.float().mean().item():.3f}")
    assert rmse <= 0.1
    assert t_plain / t_col >= 1.3


def test_hand_over_of_columns_off_the_network(ctx):
    """A batch with learned gas optics runs the learned-only kernel, which
    hands every column with a layer off the network to the full kernel.  Two
    grids -- one with columns wholly or partly off the network, one wholly on
    it -- must give, column for column, exactly what each grid gives alone;
    every column must be written; the columns wholly off the network must
    equal the plain solver's."""
    import pyoracle

    torch = _torch()
    mlp = S.load(ctx)
    sa = make_state(ProfileSpec(ncol=37, nlay=45, seed=91, t_noise=4.0, h2o_sigma=0.5))
    sb = make_state(ProfileSpec(ncol=53, nlay=45, seed=92, t_noise=4.0, h2o_sigma=0.5))
    for k in ("tlay", "tlev"):
        sa[k][:4] += 200.0          # columns 0-3: every layer off the network
    sa["tlay"][4:11, 20] += 200.0   # columns 4-10: one layer off the network
    ta, tb = pyoracle.cldprop_columns(sa), pyoracle.cldprop_columns(sb)

    def run(grids):
        mlp.batch([g.desc(seed0=s) for g, s in grids])
        torch.cuda.synchronize()
        assert ctx.sync_status() == 0
        return [g.outputs() for g, _ in grids]

    both = run([(S.DeviceGrid(sa, ta), 7), (S.DeviceGrid(sb, tb), 8)])
    alone_a = run([(S.DeviceGrid(sa, ta), 7)])[0]
    alone_b = run([(S.DeviceGrid(sb, tb), 8)])[0]
    for got, ref in ((both[0], alone_a), (both[1], alone_b)):
        for k in ref:
            assert np.array_equal(got[k], ref[k]), k
        assert (got["uflx"] > 0).all()
    gp = S.DeviceGrid(sa, ta)
    ctx.rrtmg_lw_batch_device([gp.desc(seed0=7)])
    torch.cuda.synchronize()
    plain = gp.outputs()
    for k in plain:
        assert np.array_equal(both[0][k][:4], plain[k][:4]), k
    # the partly-off columns: network layers and the taumol layer together, close to the plain solver
    d = np.abs(both[0]["uflx"][4:11] - plain["uflx"][4:11])
    assert (d <= 0.01 * np.abs(plain["uflx"][4:11]) + 5.0).all(), float(d.max())


def test_graph_of_a_learned_batch(ctx):
    """A captured batch with learned gas optics (the learned-only kernel, the
    hand-over list the graph owns, the full kernel) replays to exactly what a
    direct call gives, also when some columns are off the network."""
    import pyoracle

    torch = _torch()
    mlp = S.load(ctx)
    st = make_state(ProfileSpec(ncol=61, nlay=45, seed=93, t_noise=4.0, h2o_sigma=0.5))
    st["tlay"][5:9, 10] += 200.0  # columns 5-8: one layer off the network
    tauc = pyoracle.cldprop_columns(st)
    ga, gb = S.DeviceGrid(st, tauc), S.DeviceGrid(st, tauc)
    rows = 61 * 45
    tau = torch.empty((rows, 140), dtype=torch.float16, device="cuda")
    frac = torch.empty_like(tau)
    flag = torch.empty(rows, dtype=torch.uint8, device="cuda")
    mlp.infer(ga.desc(seed0=3), tau, frac, flag)
    sur = dict(sur_tau=tau.data_ptr(), sur_frac=frac.data_ptr(), sur_flag=flag.data_ptr())
    ctx.rrtmg_lw_batch_device([ga.desc(seed0=3, **sur)])
    graph = ctx.batch_graph([gb.desc(seed0=3, **sur)])
    try:
        graph.launch()
        graph.launch()
        torch.cuda.synchronize()
    finally:
        graph.close()
    assert ctx.sync_status() == 0
    assert flag.view(61, 45)[5:9, 10].eq(0).all()
    a, b = ga.outputs(), gb.outputs()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert (b["uflx"] > 0).all()

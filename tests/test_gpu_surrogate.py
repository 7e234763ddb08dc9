"""GPU checks of the learned wrench surrogate: each kernel against a CPU
restatement (oracle/mlp.py for the network and its gradients), the gate
routing, and an end-to-end run that trains a small network and shows what
it gains over the exact step."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import mlp  # noqa: E402
from stonefish_gb300 import abi, scenarios  # noqa: E402
from stonefish_gb300 import surrogate as S  # noqa: E402

pytestmark = pytest.mark.gpu


def _bf16(t):
    return mlp.bf16_bits_to_f32(t.contiguous().view(torch.int16).cpu().numpy())


def _dev(a, dtype=torch.float32):
    return torch.tensor(np.asarray(a), dtype=dtype, device="cuda")


def _ck(h, st):
    assert st == abi.HYDRO_OK, h.lib.hydro_last_error(h.ctx)


@pytest.mark.parametrize("epi", [0, 1, 2, 3])
def test_gemm_epilogues(hctx, epi):
    rng = np.random.default_rng(epi)
    M, N, K = 128, 192, 96
    A = mlp.bf16_round(rng.normal(size=(M, K)).astype(np.float32))
    B = mlp.bf16_round(rng.normal(size=(K, N)).astype(np.float32))
    bias = rng.normal(size=N).astype(np.float32)
    zprev = rng.normal(size=(M, N)).astype(np.float32)
    dA, dB = _dev(A, torch.bfloat16), _dev(B, torch.bfloat16)
    z = torch.zeros((M, N), dtype=torch.float32, device="cuda")
    y = torch.zeros((M, N), dtype=torch.bfloat16, device="cuda")
    db, dzp = _dev(bias), _dev(zprev)
    P = S._ptr
    _ck(hctx, hctx.lib.hydro_nn_gemm(hctx.ctx, epi, P(dA), K, P(dB), N, M, N, K, P(z), P(y), P(db), P(dzp), N,
                                     None))
    torch.cuda.synchronize()
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    if epi in (0, 2):
        r = ref + (bias if epi == 2 else 0.0)
        assert np.all(np.abs(z.cpu().numpy() - r) <= 1e-5 * (scale + np.abs(bias)) + 1e-6)
    elif epi == 1:
        r = ref + bias
        zz = z.cpu().numpy()
        assert np.all(np.abs(zz - r) <= 1e-5 * (scale + np.abs(bias)) + 1e-6)
        yy = _bf16(y)
        expect = mlp.silu(zz.astype(np.float64))
        assert np.all(np.abs(yy - expect) <= 2.0 ** -8 * np.abs(expect) + 1e-6)
    else:
        yy = _bf16(y)
        expect = ref * mlp.silu_grad(zprev.astype(np.float64))
        tol = 2.0 ** -8 * np.abs(expect) + 2e-5 * scale * np.abs(mlp.silu_grad(zprev.astype(np.float64)))
        assert np.all(np.abs(yy - expect) <= tol + 1e-6)


@pytest.mark.parametrize("M,N", [(256, 256), (64, 256), (256, 64)])
def test_weight_gradient_gemm_split_along_k(hctx, M, N):
    """The weight-gradient shapes (K = batch 4096, few output tiles) run
    split along K: the partial products are summed in slice order, so the
    result is within FP32 accumulation of the exact product and repeats
    bit for bit."""
    rng = np.random.default_rng(M + N)
    K = 4096
    A = mlp.bf16_round(rng.normal(size=(M, K)).astype(np.float32))
    B = mlp.bf16_round(rng.normal(size=(K, N)).astype(np.float32))
    dA, dB = _dev(A, torch.bfloat16), _dev(B, torch.bfloat16)
    outs = []
    for _ in range(2):
        z = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
        _ck(hctx, hctx.lib.hydro_nn_gemm(hctx.ctx, 0, S._ptr(dA), K, S._ptr(dB), N, M, N, K, S._ptr(z), None,
                                         None, None, N, None))
        torch.cuda.synchronize()
        outs.append(z.cpu().numpy())
    ref = A.astype(np.float64) @ B.astype(np.float64)
    scale = np.abs(A).astype(np.float64) @ np.abs(B).astype(np.float64)
    assert np.all(np.abs(outs[0] - ref) <= 1e-5 * scale + 1e-6)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("rows,cols", [(4096, 256), (4096, 64), (3000, 192), (256, 64)])
def test_bias_gradient_column_sums(hctx, rows, cols):
    """hydro_nn_colsum: one stage below 2048 rows, row slabs plus an in-order
    sum of the slabs above; FP32 sums of bf16 values within FP32 rounding of
    the exact sums, and the same bits on a second call."""
    rng = np.random.default_rng(rows + cols)
    g = mlp.bf16_round(rng.normal(size=(rows, cols)).astype(np.float32))
    dg = _dev(g, torch.bfloat16)
    outs = []
    for _ in range(2):
        out = torch.full((cols,), float("nan"), dtype=torch.float32, device="cuda")
        _ck(hctx, hctx.lib.hydro_nn_colsum(hctx.ctx, S._ptr(dg), rows, cols, S._ptr(out), None))
        torch.cuda.synchronize()
        outs.append(out.cpu().numpy())
    ref = g.astype(np.float64).sum(axis=0)
    scale = np.abs(g).astype(np.float64).sum(axis=0)
    assert np.all(np.abs(outs[0] - ref) <= 1e-5 * scale + 1e-6)
    assert np.array_equal(outs[0], outs[1])


def test_gemm_rejects_unaligned_shapes(hctx):
    a = torch.zeros((64, 64), dtype=torch.bfloat16, device="cuda")
    z = torch.zeros((64, 64), dtype=torch.float32, device="cuda")
    P = S._ptr
    st = hctx.lib.hydro_nn_gemm(hctx.ctx, 0, P(a), 64, P(a), 64, 64, 64, 48, P(z), None, None, None, 64, None)
    assert st == abi.HYDRO_ERR_INVALID_ARG
    st = hctx.lib.hydro_nn_gemm(hctx.ctx, 1, P(a), 64, P(a), 64, 64, 64, 64, P(z), None, None, None, 64, None)
    assert st == abi.HYDRO_ERR_INVALID_ARG   # no y / bias


def test_training_gradients_match_oracle(hctx):
    """One forward/backward pass of the full network on the GPU against the
    CPU restatement with the same bfloat16 rounding points."""
    rng = np.random.default_rng(5)
    B = 256
    sur = S.Surrogate(hctx, hidden=256, seed=3, batch=B)
    feats = _dev(rng.normal(size=(4 * B, S.N_FEAT)) * 2.0 + 1.0)
    targ = _dev(rng.normal(size=(4 * B, S.N_OUT)) * 50.0)
    sur.fit_normalisation(feats, targ)
    X = sur.prepare_inputs(feats)[:B]
    T = targ[:B]
    sur.forward_backward(X, T)
    torch.cuda.synchronize()
    x0 = _bf16(X).astype(np.float64)
    Ws = [_bf16(L["w16"]).astype(np.float64) for L in sur.layers]
    bs = [L["b"].cpu().numpy().astype(np.float64) for L in sur.layers]
    t = T.cpu().numpy()
    tn = ((t - sur.t_mean.cpu().numpy()) * sur.t_istd.cpu().numpy()).astype(np.float32).astype(np.float64)
    dWs, dbs = mlp.backward(x0, Ws, bs, tn, S.N_OUT, bf16=True)
    for l, L in enumerate(sur.layers):
        gw = L["gw"].cpu().numpy()
        gb = L["gb"].cpu().numpy()
        ew = np.linalg.norm(gw - dWs[l]) / max(np.linalg.norm(dWs[l]), 1e-30)
        eb = np.linalg.norm(gb - dbs[l]) / max(np.linalg.norm(dbs[l]), 1e-30)
        assert ew < 5e-3 and eb < 5e-3, (l, ew, eb)
    # and the bf16-free FP64 gradients agree to bfloat16 accuracy
    dW64, _ = mlp.backward(x0, Ws, bs, tn, S.N_OUT, bf16=False)
    for l in range(4):
        e = np.linalg.norm(sur.layers[l]["gw"].cpu().numpy() - dW64[l]) / np.linalg.norm(dW64[l])
        assert e < 5e-2, (l, e)


def test_adamw_step(hctx):
    rng = np.random.default_rng(2)
    rows, cols = 3, 70
    w = rng.normal(size=(rows, cols)).astype(np.float32)
    m = rng.normal(size=(rows, cols)).astype(np.float32) * 0.1
    v = np.abs(rng.normal(size=(rows, cols))).astype(np.float32) * 0.01
    g = rng.normal(size=(rows, cols)).astype(np.float32)
    dw, dm, dv, dg = _dev(w), _dev(m), _dev(v), _dev(g)
    w16 = torch.zeros((rows, cols), dtype=torch.bfloat16, device="cuda")
    wt16 = torch.zeros((cols, rows), dtype=torch.bfloat16, device="cuda")
    lr, b1, b2, eps, wd, step = 1e-2, 0.9, 0.999, 1e-8, 0.01, 7
    P = S._ptr
    _ck(hctx, hctx.lib.hydro_nn_adamw(hctx.ctx, P(dw), P(dm), P(dv), P(dg), rows, cols, cols, lr, b1, b2, eps, wd,
                                      step, P(w16), P(wt16), None))
    torch.cuda.synchronize()
    m1 = b1 * m + (1 - b1) * g
    v1 = b2 * v + (1 - b2) * g * g
    mh = m1 / (1 - b1 ** step)
    vh = v1 / (1 - b2 ** step)
    w1 = w * (1 - lr * wd) - lr * mh / (np.sqrt(vh) + eps)
    assert np.allclose(dw.cpu().numpy(), w1, rtol=1e-5, atol=1e-6)
    assert np.allclose(dm.cpu().numpy(), m1, rtol=1e-6, atol=1e-7)
    assert np.array_equal(_bf16(w16), mlp.bf16_round(dw.cpu().numpy()))
    assert np.array_equal(_bf16(wt16), mlp.bf16_round(dw.cpu().numpy()).T)


def test_features_flat_ocean(hctx):
    rng = np.random.default_rng(8)
    n = 300
    bodies = S.sample_states(rng, n)
    ocean = scenarios.flat_ocean(current=(0.2, -0.1, 0.05))
    d_b = torch.from_numpy(np.frombuffer(bodies.tobytes(), dtype=np.uint8).copy()).cuda()
    f = torch.zeros((n, 16), dtype=torch.float32, device="cuda")
    _ck(hctx, hctx.lib.hydro_nn_features(hctx.ctx, S._ptr(d_b), n, C.byref(ocean), S._ptr(f), None))
    torch.cuda.synchronize()
    f = f.cpu().numpy()
    R = bodies["T_CG"]["basis"].reshape(n, 3, 3)
    z = bodies["T_CG"]["origin"][:, 2]
    assert np.allclose(f[:, 0], z, atol=1e-6)
    assert np.allclose(f[:, 1], np.arctan2(R[:, 2, 1], R[:, 2, 2]), atol=1e-5)
    assert np.allclose(f[:, 2], np.arcsin(np.clip(-R[:, 2, 0], -1, 1)), atol=1e-5)
    vb = np.einsum("nji,nj->ni", R, bodies["v"])
    wb = np.einsum("nji,nj->ni", R, bodies["omega"])
    cb = np.einsum("nji,j->ni", R, np.array([0.2, -0.1, 0.05]))
    assert np.allclose(f[:, 3:6], vb, atol=1e-5)
    assert np.allclose(f[:, 6:9], wb, atol=1e-5)
    assert np.allclose(f[:, 9:12], cb, atol=1e-6)
    assert np.all(f[:, 12:] == 0.0)


def test_gate_and_routing(hctx):
    rng = np.random.default_rng(9)
    n = 1000
    feats = rng.normal(size=(n, 16)).astype(np.float32)
    feats[::7, 3] = 9.0                       # outside the box
    lo = np.full(16, -4.0, np.float32)
    hi = np.full(16, 4.0, np.float32)
    mean = np.zeros(16, np.float32)
    Pm = np.eye(16, dtype=np.float32)
    thr = 30.0
    mask = torch.zeros(n, dtype=torch.uint8, device="cuda")
    df = _dev(feats)
    P = S._ptr
    keep = [_dev(lo), _dev(hi), _dev(mean), _dev(Pm)]   # referenced until the kernel has run
    _ck(hctx, hctx.lib.hydro_nn_gate(hctx.ctx, P(df), n, *[P(t) for t in keep], thr, P(mask), None))
    torch.cuda.synchronize()
    inbox = np.all((feats >= lo) & (feats <= hi), axis=1)
    q = np.sum(feats.astype(np.float64) ** 2, axis=1)
    expect = inbox & (q <= thr)
    near = np.abs(q - thr) < 1e-3
    got = mask.cpu().numpy().astype(bool)
    assert np.array_equal(got[~near], expect[~near])
    assert (~got).sum() > n // 7

    # routing: rejected bodies packed in order, the rest of the slots off
    bodies = S.sample_states(rng, n)
    bodies["reserved"] = np.arange(n)
    d_b = torch.from_numpy(np.frombuffer(bodies.tobytes(), dtype=np.uint8).copy()).cuda()
    counts = torch.zeros((n + 255) // 256, dtype=torch.int32, device="cuda")
    packed = torch.zeros(n * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    pos = torch.zeros(n, dtype=torch.int32, device="cuda")
    npk = torch.zeros(1, dtype=torch.int32, device="cuda")
    _ck(hctx, hctx.lib.hydro_nn_route(hctx.ctx, P(d_b), P(mask), n, P(counts), P(packed), P(pos), P(npk), None, None))
    torch.cuda.synchronize()
    rej = np.nonzero(~got)[0]
    k = int(npk.item())
    assert k == rej.size
    pk = np.frombuffer(packed.cpu().numpy().tobytes(), dtype=abi.BODY_DTYPE)
    assert np.array_equal(pk["reserved"][:k], rej)
    assert np.all(pk["mode"][k:] == abi.MODE_DISABLED)
    p = pos.cpu().numpy()
    assert np.array_equal(p[rej], np.arange(k))
    assert np.all(p[got] == -1)
    # with an exact in-out array: its first k records zeroed, the rest untouched
    stale = torch.full((n * abi.WRENCH_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    _ck(hctx, hctx.lib.hydro_nn_route(hctx.ctx, P(d_b), P(mask), n, P(counts), P(packed), P(pos), P(npk),
                                      P(stale), None))
    torch.cuda.synchronize()
    st = stale.cpu().numpy().reshape(n, abi.WRENCH_DTYPE.itemsize)
    assert int(npk.item()) == k and np.array_equal(pos.cpu().numpy(), p)
    assert np.all(st[:k] == 0) and np.all(st[k:] == 0xAB)

    # merge: surrogate rows for accepted bodies, rotated exact wrench for the rest
    z = rng.normal(size=(n, 64)).astype(np.float32)
    ex = np.zeros(n, dtype=abi.WRENCH_DTYPE)
    for key in ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf"):
        ex[key] = rng.normal(size=(n, 3))
    d_ex = torch.from_numpy(np.frombuffer(ex.tobytes(), dtype=np.uint8).copy()).cuda()
    out = torch.zeros((n, 6), dtype=torch.float32, device="cuda")
    dz = _dev(z)
    _ck(hctx, hctx.lib.hydro_nn_merge(hctx.ctx, P(d_b), P(dz), 64, P(pos), P(d_ex), n, P(out), None))
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    assert np.array_equal(o[got], z[got, :6])
    R = bodies["T_CG"]["basis"].reshape(n, 3, 3)
    F = ex["Fb"] + ex["Fdq"] + ex["Fdf"]
    T = ex["Tb"] + ex["Tdq"] + ex["Tdf"]
    Fb = np.einsum("nji,nj->ni", R[rej], F[p[rej]])
    Tb = np.einsum("nji,nj->ni", R[rej], T[p[rej]])
    assert np.allclose(o[rej, :3], Fb, rtol=1e-6, atol=1e-5)
    assert np.allclose(o[rej, 3:], Tb, rtol=1e-6, atol=1e-5)


def test_surrogate_learns_and_beats_exact_step(built_library):
    """Trains a network on 1M states labelled by the exact step, then
    shows the gain: its wrench error is far below a constant predictor's,
    and its gated evaluation is much faster than the exact step."""
    from stonefish_gb300.hydro import HydroContext

    h64 = HydroContext(0, cut_precision=abi.CUT_FP64)
    h32 = HydroContext(0)
    xyz, fc = S.hull_mesh()
    waves = scenarios.wave_grid()
    m64, m32 = h64.upload_mesh(xyz, fc), h32.upload_mesh(xyz, fc)
    h64.set_wave_grid(waves)
    h32.set_wave_grid(waves)
    ocean, st = S.wave_ocean(), scenarios.settings()
    lab = S.Labeller(h64, m64, ocean, st)
    F, T = S.generate(lab, 1 << 20, seed=21)
    n_test = 8192
    rng = np.random.default_rng(22)
    test_bodies = S.sample_states(rng, n_test)
    Ft = torch.empty((n_test, 16), dtype=torch.float32, device="cuda")
    Tt = torch.empty((n_test, 6), dtype=torch.float32, device="cuda")
    lab.label(test_bodies, Ft, Tt)
    sur = S.Surrogate(h32, batch=1024)
    info = sur.fit(F, T, epochs=4, lr=1e-3)
    assert info["loss"][-1] < 0.2 * info["loss"][0]
    tt = Tt.cpu().numpy()
    gp = S.GatedPredictor(sur, h32, m32, n_test, ocean, st)
    test_bodies["mesh"] = m32
    d_b = torch.from_numpy(np.frombuffer(test_bodies.tobytes(), dtype=np.uint8).copy()).cuda()
    out = gp.predict(d_b).cpu().numpy()
    # the same states from page-locked host memory, read in place
    h_b = torch.from_numpy(np.frombuffer(test_bodies.tobytes(), dtype=np.uint8).copy()).pin_memory()
    assert np.array_equal(gp.predict(h_b).cpu().numpy(), out)
    err = S.wrench_errors(out, tt, ocean)
    const = S.wrench_errors(np.tile(tt.mean(0), (n_test, 1)), tt, ocean)
    assert err["wrench_median"] < 0.15 * const["wrench_median"], (err, const)
    assert err["wrench_median"] < 2.5e-2, err
    assert gp.rejected() < n_test // 20

    def timed(fn, reps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    bx = h32.batch(np.full(n_test, m32, dtype=np.uint32))
    io = torch.zeros(n_test * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    t_exact = timed(lambda: bx.compute_device(d_b.data_ptr(), ocean, st, io.data_ptr(), s), 5)
    t_sur = timed(lambda: gp.predict(d_b), 10)
    assert t_sur * 5 < t_exact, (t_sur, t_exact)
    for o in (bx, gp, lab):
        o.close()
    h32.close()
    h64.close()


def test_native_training_loop_matches_step_by_step_calls(hctx):
    """hydro_nn_train (every step's kernels launched by the library) against
    the same steps called one entry point at a time: the same kernels in the
    same order, so weights, moments and bf16 copies are bit-identical."""
    rng = np.random.default_rng(41)
    n = 7 * 256 + 37
    feats = _dev(rng.normal(size=(n, S.N_FEAT)) * 1.5 + 0.5)
    targ = _dev(rng.normal(size=(n, S.N_OUT)) * 40.0 + 5.0)
    nets = []
    losses = []
    for native in (True, False):
        sur = S.Surrogate(hctx, hidden=256, seed=11, batch=256)
        sur.fit_normalisation(feats, targ)
        info = sur.fit(feats, targ, epochs=3, lr=3e-3, warmup=5, native=native)
        torch.cuda.synchronize()
        nets.append(sur)
        losses.append(info["loss"])
    a, b = nets
    assert a.step == b.step == 3 * 7
    # the epoch losses are FP64 sums of per-block atomics (their order varies)
    np.testing.assert_allclose(losses[0], losses[1], rtol=1e-12)
    for La, Lb in zip(a.layers, b.layers):
        for f in ("w", "b", "mw", "vw", "mb", "vb", "w16", "wt16"):
            assert torch.equal(La[f], Lb[f]), f
    # a batch past the end of the inputs is rejected before anything runs
    net = a._net()
    X = a.prepare_inputs(feats)
    rows = np.array([n - 255], dtype=np.int64)
    lrs = np.array([1e-3], dtype=np.float32)
    st = hctx.lib.hydro_nn_train(hctx.ctx, C.byref(net), S._ptr(X), S._ptr(targ), n, rows.ctypes.data,
                                 lrs.ctypes.data, 1, 0, 0.9, 0.999, 1e-8, 1e-5, None)
    assert st == abi.HYDRO_ERR_INVALID_ARG
    assert torch.equal(a.layers[0]["w"], b.layers[0]["w"])


@pytest.mark.parametrize("n", [1000, 4096])
def test_fused_tensor_core_inference_matches_gemm_path(hctx, n):
    """hydro_nn_mlp_tc (tcgen05, one kernel) against the four mma.sync GEMMs:
    same BF16 weights and activations, so only the FP32 accumulation order
    and the SiLU evaluation differ."""
    rng = np.random.default_rng(31)
    sur = S.Surrogate(hctx, hidden=256, seed=7, batch=256)
    feats = _dev(rng.normal(size=(n, S.N_FEAT)) * 1.5 + 0.5)
    targ = _dev(rng.normal(size=(n, S.N_OUT)) * 40.0 + 5.0)
    sur.fit_normalisation(feats, targ)
    # a few training steps so that every layer has non-trivial weights
    sur.fit(feats[: 4 * 256].contiguous(), targ[: 4 * 256].contiguous(), epochs=2, lr=3e-3, warmup=1)
    ref = sur.infer_features(feats)[:n, :6].cpu().numpy()
    tcw = sur.tc_weights()
    out = torch.zeros(((n + 127) // 128 * 128, 16), dtype=torch.float32, device="cuda")
    got = sur.infer_tc(feats, out, tcw)[:n, :6].cpu().numpy()
    assert int(tcw["err"].item()) == 0
    scale = np.max(np.abs(ref), axis=0)
    err = np.max(np.abs(got - ref), axis=0) / scale
    assert np.all(err < 1e-2), err
    med = np.median(np.abs(got - ref), axis=0) / scale
    assert np.all(med < 1e-3), med
    assert np.all(out[n:].cpu().numpy() == 0.0)      # rows past n are not written


def _oracle_tc_forward(x_norm_bf16, Ws_bf16, bs, silu_rounding=True):
    """oracle/mlp.py's forward with the fused kernel's rounding points: BF16
    inputs and weights, FP32 pre-activations, BF16 hidden activations, FP32
    output.  Returns (a1, a2, a3, out), a_l the BF16 output of hidden layer l."""
    zs, acts = mlp.forward(x_norm_bf16, Ws_bf16, bs, bf16=True)
    return acts[1], acts[2], acts[3], zs[3]


def _pack_image(hctx, Wt_bf16):
    """The kernel's operand image from four transposed BF16 weight matrices
    (W0^T 256 x 16 padded to K 64, W1^T, W2^T 256 x 256, W3^T 16 x 256)."""
    img = torch.zeros(S.TC_IMAGE_BYTES, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for Wt, off, kpad in zip(Wt_bf16, (0, 32768, 163840, 294912), (64, 256, 256, 256)):
        t = _dev(Wt, torch.bfloat16).contiguous()
        rows, K = t.shape
        _ck(hctx, hctx.lib.hydro_nn_pack_sw128(hctx.ctx, C.c_void_p(t.data_ptr()), rows, K, K, kpad,
                                               C.c_void_p(img.data_ptr() + off), s))
    torch.cuda.synchronize()
    return img


def _run_tc(hctx, feats, fmean, fistd, img, biases):
    n = feats.shape[0]
    out = torch.zeros(((n + 127) // 128 * 128, 16), dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    b = [_dev(x) for x in biases]
    _ck(hctx, hctx.lib.hydro_nn_mlp_tc(hctx.ctx, C.c_void_p(feats.data_ptr()), n, C.c_void_p(fmean.data_ptr()),
                                       C.c_void_p(fistd.data_ptr()), C.c_void_p(img.data_ptr()),
                                       *[C.c_void_p(x.data_ptr()) for x in b], C.c_void_p(out.data_ptr()),
                                       C.c_void_p(err.data_ptr()), torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out[:n].cpu().numpy()


def _random_net(rng, H=256):
    Ws = [rng.uniform(-1, 1, (16, H)) * np.sqrt(3.0 / 16), rng.uniform(-1, 1, (H, H)) * np.sqrt(3.0 / H),
          rng.uniform(-1, 1, (H, H)) * np.sqrt(3.0 / H)]
    bs = [rng.normal(size=H) * 0.3 for _ in range(3)]
    return [mlp.bf16_round(w.astype(np.float32)) for w in Ws], [b.astype(np.float32) for b in bs]


@pytest.mark.parametrize("n", [1000, 65536])
def test_fused_tensor_core_kernel_against_oracle_layers(hctx, n):
    """The shipped inference kernel (hydro_nn_mlp_tc) against oracle/mlp.py
    with the same BF16 rounding points.  The last layer is set to select 16
    of the 256 third-layer activations (weights 1, bias 0: one exact product
    each), so the kernel's output is those activations themselves; two runs
    observe columns 0-15 and 240-255.  Each activation may differ from the
    oracle's by the BF16 roundings that the FP32 summation order and the
    kernel's tanh-based SiLU move across a rounding boundary: per layer at
    most one BF16 step (2^-8 of the value), and over three layers the bar is
    2^-6 of max(|a|, the row's RMS), with the median under 2^-10.  n = 1000
    is not a multiple of the kernel's 128-row block; 65536 is the benchmark
    batch (checked on 4096 of its rows)."""
    rng = np.random.default_rng(41)
    Ws, bs = _random_net(rng)
    f = (rng.normal(size=(n, 16)) * 1.5 + 0.5).astype(np.float32)
    fmean = rng.normal(size=16).astype(np.float32) * 0.2
    fistd = rng.uniform(0.5, 1.5, 16).astype(np.float32)
    x = mlp.bf16_round((f - fmean) * fistd)
    rows = np.arange(n) if n <= 4096 else np.sort(rng.choice(n, 4096, replace=False))
    a1, a2, a3, _ = _oracle_tc_forward(x[rows], Ws + [np.zeros((256, 16), np.float32)], bs + [np.zeros(16)])
    feats, dm, di = _dev(f), _dev(fmean), _dev(fistd)
    for first in (0, 240):
        W3 = np.zeros((256, 16), np.float32)
        W3[first + np.arange(16), np.arange(16)] = 1.0
        img = _pack_image(hctx, [np.ascontiguousarray(W.T) for W in Ws + [W3]])
        got = _run_tc(hctx, feats, dm, di, img, bs + [np.zeros(16, np.float32)])[rows]
        ref = a3[:, first:first + 16]
        scale = np.maximum(np.abs(ref), np.sqrt(np.mean(a3 * a3, axis=1, keepdims=True)))
        rel = np.abs(got - ref) / scale
        assert float(rel.max()) <= 2.0 ** -6, (first, float(rel.max()))
        assert float(np.median(rel)) <= 2.0 ** -10, (first, float(np.median(rel)))


def test_fused_tensor_core_kernel_against_oracle_output(hctx):
    """The whole network as the gated predictor runs it (trained weights, the
    target de-normalisation folded into the last layer) against
    oracle/mlp.py: per output column, max error within 2^-7 and median within
    2^-10 of the column's scale."""
    rng = np.random.default_rng(43)
    n = 3000
    sur = S.Surrogate(hctx, hidden=256, seed=9, batch=256)
    feats = _dev(rng.normal(size=(n, S.N_FEAT)) * 1.5 + 0.5)
    targ = _dev(rng.normal(size=(n, S.N_OUT)) * 40.0 + 5.0)
    sur.fit_normalisation(feats, targ)
    sur.fit(feats[: 4 * 256].contiguous(), targ[: 4 * 256].contiguous(), epochs=2, lr=3e-3, warmup=1)
    tcw = sur.tc_weights()
    out = torch.zeros(((n + 127) // 128 * 128, 16), dtype=torch.float32, device="cuda")
    got = sur.infer_tc(feats, out, tcw)[:n, :6].cpu().numpy()
    # the same weights on the host, rounded where the kernel's image holds them
    Ws = [_bf16(sur.layers[l]["w16"])[:16 if l == 0 else 256, :256] for l in range(3)]
    w3 = sur.layers[3]["w"].cpu().numpy().astype(np.float64)
    w3[:, :S.N_OUT] *= sur.stats["t_std"]
    Ws.append(mlp.bf16_round(w3[:, :16].astype(np.float32)))
    bs = [sur.layers[l]["b"].cpu().numpy() for l in range(3)] + [tcw["b"][3].cpu().numpy()]
    f = feats.cpu().numpy()
    x = mlp.bf16_round((f - sur.f_mean.cpu().numpy()) * sur.f_istd.cpu().numpy())
    ref = _oracle_tc_forward(x, Ws, bs)[3][:, :6]
    scale = np.max(np.abs(ref), axis=0)
    err = np.abs(got - ref) / scale
    assert np.all(err.max(axis=0) <= 2.0 ** -7), err.max(axis=0)
    assert np.all(np.median(err, axis=0) <= 2.0 ** -10), np.median(err, axis=0)


def test_gate_inside_matches_fluid_position(built_library, oracle):
    """States whose AABB lies wholly under the wavy surface (the reference's
    INSIDE branch, SolidEntity.cpp:1239-1261) leave the network's path;
    states already rejected stay rejected and the others keep their bit."""
    from stonefish_gb300.hydro import HydroContext
    rng = np.random.default_rng(41)
    n = 2000
    waves = scenarios.wave_grid(n=256, n_waves=16, seed=3)
    ocean = S.wave_ocean()
    bodies = S.sample_states(rng, n, depth=(-1.5, 1.5), extent=25.6)
    h = HydroContext()
    try:
        h.set_wave_grid(waves)
        m0 = np.ones(n, np.uint8)
        m0[::5] = 0
        mask = torch.from_numpy(m0.copy()).cuda()
        d_b = torch.from_numpy(np.frombuffer(bodies.tobytes(), dtype=np.uint8).copy()).cuda()
        _ck(h, h.lib.hydro_nn_gate_inside(h.ctx, S._ptr(d_b), n, C.byref(ocean), S._ptr(mask), None))
        torch.cuda.synchronize()
        got = mask.cpu().numpy()
    finally:
        h.close()
    inside = np.array([oracle.fluid_position(ocean, bodies["aabb_min"][i], bodies["aabb_max"][i], waves)
                       == abi.INSIDE for i in range(n)])
    expect = (m0 != 0) & ~inside
    assert np.array_equal(got != 0, expect)
    assert inside.sum() > 50 and (~inside).sum() > 50


def test_ensemble_mean_and_disagreement_gate(hctx):
    """Two networks' outputs: the first becomes their mean (columns 0..5),
    and a state whose outputs differ by more than tau in the wrench metric
    (max of |dF| / fs and |dT| / ts) is rejected."""
    rng = np.random.default_rng(42)
    n, ld = 3000, 16
    za = rng.normal(size=(n, ld)).astype(np.float32)
    zb = (za + rng.normal(size=(n, ld)) * rng.uniform(0.0, 0.2, (n, 1))).astype(np.float32)
    m0 = np.ones(n, np.uint8)
    m0[::9] = 0
    fs, ts, tau = 3.0, 5.0, 0.05
    dza, dzb, mask = _dev(za), _dev(zb), torch.from_numpy(m0.copy()).cuda()
    _ck(hctx, hctx.lib.hydro_nn_ensemble(hctx.ctx, S._ptr(dza), S._ptr(dzb), ld, n, fs, ts, tau, S._ptr(mask), None))
    torch.cuda.synchronize()
    out = dza.cpu().numpy()
    mean = ((za + zb) * np.float32(0.5)).astype(np.float32)
    assert np.array_equal(out[:, :6], mean[:, :6])
    assert np.array_equal(out[:, 6:], za[:, 6:])
    d = np.maximum(np.linalg.norm(za[:, :3].astype(np.float64) - zb[:, :3], axis=1) / fs,
                   np.linalg.norm(za[:, 3:6].astype(np.float64) - zb[:, 3:6], axis=1) / ts)
    clear = np.abs(d - tau) > 1e-5
    expect = (m0 != 0) & (d <= tau)
    got = mask.cpu().numpy() != 0
    assert np.array_equal(got[clear], expect[clear])
    assert (~expect & (m0 != 0)).sum() > 100 and expect.sum() > 100


def test_audit_pick_and_error(hctx):
    """The audit sends rows phase, phase + stride, ... that the gates
    admitted to the exact step and measures the network's error on them
    against the exact wrench rotated into the body frame."""
    rng = np.random.default_rng(43)
    n, stride, phase = 5000, 64, 17
    k = (n + stride - 1) // stride
    m0 = (rng.uniform(size=n) > 0.3).astype(np.uint8)
    mask = torch.from_numpy(m0.copy()).cuda()
    idx = torch.zeros(k, dtype=torch.int32, device="cuda")
    _ck(hctx, hctx.lib.hydro_nn_audit_pick(hctx.ctx, S._ptr(mask), n, stride, phase, k, S._ptr(idx), None))
    torch.cuda.synchronize()
    rows = phase + stride * np.arange(k)
    want = np.where((rows < n) & (m0[np.minimum(rows, n - 1)] != 0), rows, -1)
    got_idx = idx.cpu().numpy()
    assert np.array_equal(got_idx, want)
    m1 = m0.copy()
    m1[want[want >= 0]] = 0
    assert np.array_equal(mask.cpu().numpy(), m1)
    # errors: picked rows take slots of an exact array, one picked row is
    # left without a slot (its error slot reads -1, as empty sample slots do)
    bodies = S.sample_states(rng, n)
    picked = want[want >= 0]
    pos = np.full(n, -1, np.int32)
    pos[picked[1:]] = np.arange(picked.size - 1)
    ex = np.zeros(n, dtype=abi.WRENCH_DTYPE)
    for key in ("Fb", "Tb", "Fdq", "Tdq", "Fdf", "Tdf"):
        ex[key] = rng.normal(size=(n, 3))
    z = rng.normal(size=(n, 16)).astype(np.float32)
    fs, ts = 2.0, 3.0
    err = torch.zeros(k, dtype=torch.float32, device="cuda")
    d_b = torch.from_numpy(np.frombuffer(bodies.tobytes(), dtype=np.uint8).copy()).cuda()
    d_ex = torch.from_numpy(np.frombuffer(ex.tobytes(), dtype=np.uint8).copy()).cuda()
    dz, dpos = _dev(z), torch.from_numpy(pos).cuda()
    _ck(hctx, hctx.lib.hydro_nn_audit_error(hctx.ctx, S._ptr(d_b), S._ptr(dz), 16, S._ptr(dpos), S._ptr(d_ex),
                                            S._ptr(idx), k, fs, ts, S._ptr(err), None))
    torch.cuda.synchronize()
    e = err.cpu().numpy()
    R = bodies["T_CG"]["basis"].reshape(n, 3, 3)
    F = ex["Fb"] + ex["Fdq"] + ex["Fdf"]
    T = ex["Tb"] + ex["Tdq"] + ex["Tdf"]
    for j, i in enumerate(want):
        if i < 0 or pos[i] < 0:
            assert e[j] == -1.0
            continue
        Fb = R[i].T @ F[pos[i]]
        Tb = R[i].T @ T[pos[i]]
        x = max(np.linalg.norm(z[i, :3] - Fb) / fs, np.linalg.norm(z[i, 3:6] - Tb) / ts)
        assert abs(e[j] - x) <= 1e-6 * x + 1e-7
    assert (e > 0).sum() >= picked.size - 1

"""Learned wrench surrogate for one fixed hull, with an out-of-distribution
gate that sends unfamiliar states to the exact integrator.

Nothing here has a counterpart in the reference: Stonefish integrates every
face of every body at every hydrodynamics tick
(SolidEntity::ComputeHydrodynamicForces, SolidEntity.cpp:1799-1850).  This
module adds a cheaper path for a hull that is simulated many times over:

* ``generate``: states drawn uniformly over the training domain are
  labelled by the exact step (FP32 face arithmetic, FP64 cut points and
  sums) and turned into 16 features (``hydro_nn_features``) and a body-frame
  6-DoF wrench target (``hydro_nn_wrench_body``);
* ``Surrogate``: an MLP 16 -> 256 -> 256 -> 256 -> 6 with SiLU activations,
  BF16 weights and activations and FP32 accumulation, trained by the
  library's own kernels (tensor-core GEMMs with fused bias/SiLU epilogues,
  MSE gradient, bias-gradient column sums, AdamW on FP32 master weights);
* ``Surrogate.predict``: features -> gate -> normalised BF16 input -> four
  GEMMs -> the gate's rejects packed into an exact step -> merge.

Device memory comes from torch tensors (allocation and zeroing only); every
computation is a call into the C ABI.  The error of a predicted wrench is
measured against the full-immersion scale of the hull: force error
|dF| / (rho g V) and torque error |dT| / (rho g V L/2), L the hull length.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import abi, meshes, scenarios
from .hydro import HydroContext, _check

N_FEAT = 16
N_OUT = 6
IN_PAD = 64          # input columns (features padded; GEMM tiles are 64 wide)
TC_IMAGE_BYTES = 303104   # HYDRO_NN_TC_IMAGE_BYTES
OUT_PAD = 64         # output columns (6 used)

# the training hull: the torpedo of the wave workload at 12000 faces
HULL_RADIUS = 0.25
HULL_LENGTH = 2.0
HULL_FACES = 12000
HULL_CD = (1.0, 0.5, 0.5)
HULL_CF = (0.1, 0.05, 0.05)


def _ptr(t) -> C.c_void_p | None:
    return None if t is None else C.c_void_p(t.data_ptr())


def hull_mesh(faces: int = HULL_FACES):
    return meshes.capped_cylinder_for_faces(HULL_RADIUS, HULL_LENGTH, faces)


def hull_scales(ocean: abi.Ocean) -> tuple[float, float]:
    """(force scale rho g V, torque scale rho g V L_total/2) of the hull."""
    vol = meshes.capped_cylinder_volume(HULL_RADIUS, HULL_LENGTH)
    fs = ocean.density * ocean.gravity * vol
    return fs, fs * (0.5 * HULL_LENGTH + HULL_RADIUS)


def sample_states(rng: np.random.Generator, n: int, depth=(-1.0, 0.3), extent: float = 102.4,
                  v_range: float = 1.0, w_range: float = 0.5, surface=None, w_body=None) -> np.ndarray:
    """Hull states drawn uniformly: CG x, y over the wave grid, CG z in
    ``depth`` (below the local surface when ``surface(xy) -> z`` is given,
    else absolute), uniform random orientation, v in [-v_range, v_range]^3,
    omega in [-w_range, w_range]^3 (the defaults are the single-body and
    wave workloads' ranges), or, with ``w_body`` = (a, b, c), omega drawn in
    the body frame from [-a, a] x [-b, b] x [-c, c] (a free hull spins
    about its long axis much faster than it pitches or yaws).  Returns a
    hydro_body array with mesh id 0."""
    q = scenarios.random_quaternions(rng, n)
    R = scenarios.quat_to_matrix(q)
    pos = np.empty((n, 3))
    pos[:, 0] = rng.uniform(0.0, extent, n)
    pos[:, 1] = rng.uniform(0.0, extent, n)
    pos[:, 2] = rng.uniform(depth[0], depth[1], n)
    if surface is not None:
        pos[:, 2] += surface(pos[:, :2])
    v = rng.uniform(-v_range, v_range, (n, 3))
    if w_body is None:
        w = rng.uniform(-w_range, w_range, (n, 3))
    else:
        wb = rng.uniform(-1.0, 1.0, (n, 3)) * np.asarray(w_body, dtype=np.float64)
        w = np.einsum("nij,nj->ni", R, wb)
    half = np.tile([0.5 * HULL_LENGTH + HULL_RADIUS, HULL_RADIUS, HULL_RADIUS], (n, 1))
    return scenarios.fill_bodies(n, R, pos, v, w, half,
                                 meshes.capped_cylinder_volume(HULL_RADIUS, HULL_LENGTH),
                                 meshes.capped_cylinder_surface(HULL_RADIUS, HULL_LENGTH),
                                 HULL_CD, HULL_CF, 0)


def wave_ocean() -> abi.Ocean:
    o = scenarios.flat_ocean()
    o.waves = 1
    return o


class Labeller:
    """Runs the exact step over chunks of hull states and produces features
    and body-frame wrench targets on the device."""

    def __init__(self, hctx: HydroContext, mesh_id: int, ocean: abi.Ocean, settings: abi.Settings,
                 chunk: int = 65536):
        self.h = hctx
        self.lib = hctx.lib
        self.ocean = ocean
        self.settings = settings
        self.chunk = chunk
        self.mesh_id = mesh_id
        self.dev = torch.device("cuda", hctx.device)
        self.batch = hctx.batch(np.full(chunk, mesh_id, dtype=np.uint32))
        self.d_bodies = torch.empty(chunk * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, device=self.dev)
        self.d_io = torch.zeros(chunk * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device=self.dev)
        self.h_bodies = torch.empty(chunk * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)

    def _ck(self, st):
        _check(self.lib, self.h.ctx, st)

    def label(self, bodies: np.ndarray, feats: torch.Tensor, targets: torch.Tensor,
              wrenches: torch.Tensor | None = None) -> None:
        """bodies: host hydro_body[n <= chunk]; writes feats[n,16], targets[n,6]
        (device float32) and, when given, the raw wrenches (device bytes)."""
        n = bodies.size
        assert n <= self.chunk
        b = bodies.copy()
        b["mesh"] = self.mesh_id
        # the pinned staging buffer may still feed the previous chunk's copy
        torch.cuda.current_stream(self.dev).synchronize()
        hb = self.h_bodies.numpy()[: b.nbytes]
        hb[:] = np.frombuffer(b.tobytes(), dtype=np.uint8)
        if n < self.chunk:
            # the batch always spans `chunk` bodies; the tail is switched off
            self.d_bodies.zero_()
        self.d_bodies[: b.nbytes].copy_(self.h_bodies[: b.nbytes], non_blocking=True)
        self.d_io.zero_()
        s = torch.cuda.current_stream(self.dev).cuda_stream
        self.batch.compute_device(self.d_bodies.data_ptr(), self.ocean, self.settings,
                                  self.d_io.data_ptr(), s)
        self._ck(self.lib.hydro_nn_wrench_body(self.h.ctx, _ptr(self.d_bodies), _ptr(self.d_io), n,
                                               _ptr(targets), s))
        self._ck(self.lib.hydro_nn_features(self.h.ctx, _ptr(self.d_bodies), n, C.byref(self.ocean),
                                            _ptr(feats), s))
        if wrenches is not None:
            wrenches[: n * abi.WRENCH_DTYPE.itemsize].copy_(self.d_io[: n * abi.WRENCH_DTYPE.itemsize])

    def close(self):
        self.batch.close()


def generate(labeller: Labeller, n: int, seed: int, **state_ranges):
    """n labelled samples: (features [n,16], targets [n,6]) device tensors."""
    dev = labeller.dev
    feats = torch.empty((n, N_FEAT), dtype=torch.float32, device=dev)
    targ = torch.empty((n, N_OUT), dtype=torch.float32, device=dev)
    rng = np.random.default_rng(seed)
    for off in range(0, n, labeller.chunk):
        m = min(labeller.chunk, n - off)
        labeller.label(sample_states(rng, m, **state_ranges), feats[off:off + m], targ[off:off + m])
    return feats, targ


class Surrogate:
    """The MLP, its optimiser state, normalisation and gate."""

    def __init__(self, hctx: HydroContext, hidden: int = 256, seed: int = 0, batch: int = 4096):
        assert hidden % 64 == 0 and batch % 64 == 0
        self.h = hctx
        self.lib = hctx.lib
        self.dev = torch.device("cuda", hctx.device)
        self.hidden = hidden
        self.B = batch
        dims = [(IN_PAD, hidden), (hidden, hidden), (hidden, hidden), (hidden, OUT_PAD)]
        fan = [N_FEAT, hidden, hidden, hidden]
        rng = np.random.default_rng(seed)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.layers = []
        for l, (k, n) in enumerate(dims):
            w = np.zeros((k, n), dtype=np.float32)
            kr = fan[l]
            nr = N_OUT if l == 3 else n
            w[:kr, :nr] = rng.uniform(-1.0, 1.0, (kr, nr)) * math.sqrt(3.0 / kr)
            L = {
                "k": k, "n": n,
                "w": torch.from_numpy(w).to(self.dev),
                "b": torch.zeros(n, **f32),
                "mw": torch.zeros((k, n), **f32), "vw": torch.zeros((k, n), **f32),
                "mb": torch.zeros(n, **f32), "vb": torch.zeros(n, **f32),
                "gw": torch.zeros((k, n), **f32), "gb": torch.zeros(n, **f32),
                "w16": torch.zeros((k, n), dtype=torch.bfloat16, device=self.dev),
                "wt16": torch.zeros((n, k), dtype=torch.bfloat16, device=self.dev),
            }
            self.layers.append(L)
        self._refresh_bf16()
        self.step = 0
        self.loss_d = torch.zeros(1, dtype=torch.float64, device=self.dev)
        self.f_mean = self.f_istd = self.t_mean = self.t_istd = None
        self.gate = None
        self._train_bufs = None
        self._infer = {}

    # ----------------------------------------------------------- plumbing
    def _ck(self, st):
        _check(self.lib, self.h.ctx, st)

    def _s(self):
        return torch.cuda.current_stream(self.dev).cuda_stream

    def gemm(self, epi, A, lda, B, ldb, M, N, K, z=None, y=None, bias=None, zprev=None, ldc=None):
        self._ck(self.lib.hydro_nn_gemm(self.h.ctx, epi, _ptr(A), lda, _ptr(B), ldb, M, N, K, _ptr(z),
                                        _ptr(y), _ptr(bias), _ptr(zprev), ldc or N, self._s()))

    def to_bf16(self, x, rows, n_in, ld, y, mean=None, istd=None):
        self._ck(self.lib.hydro_nn_to_bf16(self.h.ctx, _ptr(x), rows, n_in, ld, _ptr(mean), _ptr(istd),
                                           _ptr(y), self._s()))

    def _refresh_bf16(self):
        for L in self.layers:
            self.to_bf16(L["w"], L["k"], L["n"], L["n"], L["w16"])
            self._ck(self.lib.hydro_nn_transpose(self.h.ctx, _ptr(L["w16"]), _ptr(L["wt16"]), L["k"], L["n"],
                                                 self._s()))

    # ------------------------------------------------------ normalisation
    def fit_normalisation(self, feats: torch.Tensor, targets: torch.Tensor, sample: int = 1 << 20,
                          gate_quantile: float = 0.999, box_margin: float = 0.02,
                          target_scales: tuple[float, ...] | None = None) -> None:
        """Feature/target statistics and the gate, from up to ``sample`` rows
        (host FP64 arithmetic on a copy).  Targets are centred and divided by
        their standard deviations, or, with ``target_scales`` = (force scale,
        torque scale), by those two scales: the training loss then weighs
        each component's error as the wrench error metric does.  Six scales
        (one per component) weigh the components individually."""
        f = feats[:sample].double().cpu().numpy()
        t = targets[:sample].double().cpu().numpy()
        fm, fs = f.mean(0), f.std(0)
        fs[fs < 1e-12] = 1.0
        tm, ts = t.mean(0), t.std(0)
        ts[ts < 1e-12] = 1.0
        if target_scales is not None:
            if len(target_scales) == 6:
                ts = np.array(target_scales, dtype=np.float64)
            else:
                ts = np.array([target_scales[0]] * 3 + [target_scales[1]] * 3, dtype=np.float64)
        f32 = dict(dtype=torch.float32, device=self.dev)
        self.f_mean = torch.tensor(fm, **f32)
        self.f_istd = torch.tensor(1.0 / fs, **f32)
        self.t_mean = torch.tensor(tm, **f32)
        self.t_istd = torch.tensor(1.0 / ts, **f32)
        self.stats = {"f_mean": fm, "f_std": fs, "t_mean": tm, "t_std": ts}
        # gate: per-feature box widened by box_margin of the range, plus a
        # Mahalanobis radius at the gate_quantile of the training sample
        lo, hi = f.min(0), f.max(0)
        span = np.maximum(hi - lo, 1e-6)
        lo, hi = lo - box_margin * span, hi + box_margin * span
        cov = np.cov(f, rowvar=False) + np.eye(N_FEAT) * 1e-9
        P = np.linalg.inv(cov)
        d = f - fm
        q = np.einsum("ij,jk,ik->i", d, P, d)
        thr = float(np.quantile(q, gate_quantile))
        self.gate = {
            "lo": torch.tensor(lo, **f32), "hi": torch.tensor(hi, **f32),
            "mean": torch.tensor(fm, **f32), "P": torch.tensor(P, **f32), "thr": thr,
        }

    # -------------------------------------------------------------- train
    def _bufs(self):
        if self._train_bufs is None:
            B, H = self.B, self.hidden
            bf = dict(dtype=torch.bfloat16, device=self.dev)
            f32 = dict(dtype=torch.float32, device=self.dev)
            self._train_bufs = {
                "z": [torch.empty((B, H), **f32) for _ in range(3)] + [torch.empty((B, OUT_PAD), **f32)],
                "x": [torch.empty((B, H), **bf) for _ in range(3)],
                "dz": [torch.empty((B, H), **bf) for _ in range(3)] + [torch.empty((B, OUT_PAD), **bf)],
                "xt": [torch.empty((IN_PAD, B), **bf)] + [torch.empty((H, B), **bf) for _ in range(3)],
            }
        return self._train_bufs

    def forward_backward(self, X0: torch.Tensor, T: torch.Tensor) -> None:
        """One forward and backward pass on a batch: X0 [B,64] bf16
        (normalised, padded), T [B,6] raw targets.  Leaves gw/gb per layer."""
        B, H = self.B, self.hidden
        bf = self._bufs()
        z, x, dz, xt = bf["z"], bf["x"], bf["dz"], bf["xt"]
        Ls = self.layers
        ins = [X0, x[0], x[1], x[2]]
        for l in range(3):
            self.gemm(1, ins[l], Ls[l]["k"], Ls[l]["w16"], Ls[l]["n"], B, H, Ls[l]["k"],
                      z=z[l], y=x[l], bias=Ls[l]["b"])
        self.gemm(2, x[2], H, Ls[3]["w16"], OUT_PAD, B, OUT_PAD, H, z=z[3], bias=Ls[3]["b"])
        self._ck(self.lib.hydro_nn_mse_grad(self.h.ctx, _ptr(z[3]), _ptr(T), B, OUT_PAD, N_OUT,
                                            _ptr(self.t_mean), _ptr(self.t_istd), _ptr(dz[3]),
                                            _ptr(self.loss_d), self._s()))
        for l in range(3, -1, -1):
            L = Ls[l]
            k = L["k"]
            self._ck(self.lib.hydro_nn_transpose(self.h.ctx, _ptr(ins[l]), _ptr(xt[l]), B, k, self._s()))
            self.gemm(0, xt[l], B, dz[l], L["n"], k, L["n"], B, z=L["gw"])
            self._ck(self.lib.hydro_nn_colsum(self.h.ctx, _ptr(dz[l]), B, L["n"], _ptr(L["gb"]), self._s()))
            if l > 0:
                self.gemm(3, dz[l], L["n"], L["wt16"], k, B, k, L["n"], y=dz[l - 1], zprev=z[l - 1])

    def optimizer_step(self, lr: float, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-5) -> None:
        self.step += 1
        for L in self.layers:
            self._ck(self.lib.hydro_nn_adamw(self.h.ctx, _ptr(L["w"]), _ptr(L["mw"]), _ptr(L["vw"]),
                                             _ptr(L["gw"]), L["k"], L["n"], L["n"], lr, beta1, beta2, eps,
                                             weight_decay, self.step, _ptr(L["w16"]), _ptr(L["wt16"]),
                                             self._s()))
            self._ck(self.lib.hydro_nn_adamw(self.h.ctx, _ptr(L["b"]), _ptr(L["mb"]), _ptr(L["vb"]),
                                             _ptr(L["gb"]), 1, L["n"], L["n"], lr, beta1, beta2, eps,
                                             0.0, self.step, None, None, self._s()))
        self._infer.clear()

    def prepare_inputs(self, feats: torch.Tensor) -> torch.Tensor:
        """Normalised, padded BF16 network inputs [n,64] for feature rows."""
        n = feats.shape[0]
        X = torch.empty((n, IN_PAD), dtype=torch.bfloat16, device=self.dev)
        self.to_bf16(feats, n, N_FEAT, IN_PAD, X, self.f_mean, self.f_istd)
        return X

    def _net(self) -> abi.NnNet:
        """The network and the training buffers as hydro_nn_train reads them."""
        bf = self._bufs()
        net = abi.NnNet()
        for l, L in enumerate(self.layers):
            d = net.layer[l]
            for f in ("w", "b", "mw", "vw", "mb", "vb", "gw", "gb", "w16", "wt16"):
                setattr(d, f, L[f].data_ptr())
            d.k, d.n = L["k"], L["n"]
        for l in range(4):
            net.z[l] = bf["z"][l].data_ptr()
            net.dz[l] = bf["dz"][l].data_ptr()
            net.xt[l] = bf["xt"][l].data_ptr()
        for l in range(3):
            net.x[l] = bf["x"][l].data_ptr()
        net.tmean, net.tistd = self.t_mean.data_ptr(), self.t_istd.data_ptr()
        net.loss = self.loss_d.data_ptr()
        net.batch, net.n_out = self.B, N_OUT
        return net

    def fit(self, feats: torch.Tensor, targets: torch.Tensor, epochs: int = 4, lr: float = 2e-3,
            lr_final: float = 2e-5, warmup: int = 200, log=None, on_epoch=None, native: bool = True) -> dict:
        """AdamW with linear warm-up and cosine decay over ``epochs`` passes
        of consecutive batches (samples are i.i.d., so no shuffling is
        needed; each epoch shifts the batch boundaries).  With ``native``
        each epoch is one hydro_nn_train call (the library launches every
        step's kernels); otherwise the same kernels are called step by step
        from here, with the same result bits."""
        if self.f_mean is None:
            self.fit_normalisation(feats, targets)
        X = self.prepare_inputs(feats)
        T = targets.contiguous()
        n = feats.shape[0] // self.B * self.B
        if n == 0:
            raise ValueError(f"fit needs at least one batch of {self.B} rows, got {feats.shape[0]}")
        per_epoch = n // self.B
        total = epochs * per_epoch
        history = []
        net = self._net() if native else None
        torch.cuda.synchronize(self.dev)
        t0 = time.perf_counter()
        it = 0
        for e in range(epochs):
            shift = (e * 997) % (feats.shape[0] - n + 1)
            self.loss_d.zero_()
            rows = np.empty(per_epoch, dtype=np.int64)
            lrs = np.empty(per_epoch, dtype=np.float32)
            for i in range(per_epoch):
                rows[i] = shift + i * self.B
                g = (it + i) / max(total - 1, 1)
                cur = lr_final + 0.5 * (lr - lr_final) * (1.0 + math.cos(math.pi * g))
                if it + i < warmup:
                    cur *= (it + i + 1) / warmup
                lrs[i] = cur
            if native:
                self._ck(self.lib.hydro_nn_train(self.h.ctx, C.byref(net), _ptr(X), _ptr(T), feats.shape[0],
                                                 rows.ctypes.data, lrs.ctypes.data, per_epoch, self.step,
                                                 0.9, 0.999, 1e-8, 1e-5, self._s()))
                self.step += per_epoch
                self._infer.clear()
            else:
                for i in range(per_epoch):
                    a = int(rows[i])
                    self.forward_backward(X[a:a + self.B], T[a:a + self.B])
                    self.optimizer_step(float(lrs[i]))
            it += per_epoch
            mean_loss = float(self.loss_d.item()) / per_epoch
            history.append(mean_loss)
            if log:
                log(f"epoch {e}: loss {mean_loss:.3e} ({time.perf_counter() - t0:.1f} s)")
            if on_epoch:
                on_epoch(e)
        torch.cuda.synchronize(self.dev)
        return {"loss": history, "seconds": time.perf_counter() - t0, "steps": total,
                "samples_per_s": total * self.B / (time.perf_counter() - t0)}

    # ---------------------------------------------------------- inference
    def _fold_output(self):
        """Inference copy of the last layer with the target de-normalisation
        folded in: W' = W diag(std), b' = b std + mean."""
        L = self.layers[3]
        w = L["w"].cpu().numpy().astype(np.float64)
        b = L["b"].cpu().numpy().astype(np.float64)
        std, mean = self.stats["t_std"], self.stats["t_mean"]
        w[:, :N_OUT] *= std
        b[:N_OUT] = b[:N_OUT] * std + mean
        wf = torch.tensor(w, dtype=torch.float32, device=self.dev)
        w16 = torch.empty((L["k"], L["n"]), dtype=torch.bfloat16, device=self.dev)
        self.to_bf16(wf, L["k"], L["n"], L["n"], w16)
        return w16, torch.tensor(b, dtype=torch.float32, device=self.dev)

    def _infer_bufs(self, n_pad: int):
        key = n_pad
        if key not in self._infer:
            H = self.hidden
            bf = dict(dtype=torch.bfloat16, device=self.dev)
            w16, b = self._fold_output()
            self._infer[key] = {
                "feats": torch.zeros((n_pad, N_FEAT), dtype=torch.float32, device=self.dev),
                "X0": torch.zeros((n_pad, IN_PAD), **bf),
                "x": [torch.empty((n_pad, H), **bf) for _ in range(3)],
                "z": torch.empty((n_pad, OUT_PAD), dtype=torch.float32, device=self.dev),
                "mask": torch.zeros(n_pad, dtype=torch.uint8, device=self.dev),
                "w3": w16, "b3": b,
            }
        return self._infer[key]

    def infer_features(self, feats: torch.Tensor, out_z: torch.Tensor | None = None) -> torch.Tensor:
        """Network outputs (de-normalised body-frame wrench) for feature rows,
        no gate: returns z [n_pad, 64] (columns 0..5 used)."""
        n = feats.shape[0]
        n_pad = (n + 63) // 64 * 64
        bufs = self._infer_bufs(n_pad)
        self.to_bf16(feats, n, N_FEAT, IN_PAD, bufs["X0"], self.f_mean, self.f_istd)
        self._mlp(bufs, n_pad)
        return bufs["z"]

    def tc_weights(self) -> dict:
        """Weights of the fused tensor-core kernel (hydro_nn_mlp_tc): the four
        layers' transposes in the 128-byte-swizzled operand image, the last
        layer with the target de-normalisation folded in and its output
        padded to 16 columns, and the biases."""
        L = self.layers
        img = torch.zeros(TC_IMAGE_BYTES, dtype=torch.uint8, device=self.dev)
        st = self._s()
        offs = (0, 32768, 163840)
        for l in range(3):
            self._ck(self.lib.hydro_nn_pack_sw128(self.h.ctx, _ptr(L[l]["wt16"]), L[l]["n"], L[l]["k"], L[l]["k"],
                                                  L[l]["k"], C.c_void_p(img.data_ptr() + offs[l]), st))
        w = L[3]["w"].cpu().numpy().astype(np.float64)
        b = L[3]["b"].cpu().numpy().astype(np.float64)
        std, mean = self.stats["t_std"], self.stats["t_mean"]
        w[:, :N_OUT] *= std
        b[:N_OUT] = b[:N_OUT] * std + mean
        w3t = torch.tensor(np.ascontiguousarray(w[:, :16].T), dtype=torch.float32, device=self.dev)
        w3t16 = torch.empty((16, self.hidden), dtype=torch.bfloat16, device=self.dev)
        self.to_bf16(w3t, 16, self.hidden, self.hidden, w3t16)
        self._ck(self.lib.hydro_nn_pack_sw128(self.h.ctx, _ptr(w3t16), 16, self.hidden, self.hidden, self.hidden,
                                              C.c_void_p(img.data_ptr() + 294912), st))
        torch.cuda.synchronize(self.dev)
        return {"image": img, "b": [L[0]["b"].clone(), L[1]["b"].clone(), L[2]["b"].clone(),
                                    torch.tensor(b[:16], dtype=torch.float32, device=self.dev)],
                "err": torch.zeros(1, dtype=torch.int32, device=self.dev)}

    def infer_tc(self, feats: torch.Tensor, out: torch.Tensor, tcw: dict) -> torch.Tensor:
        """Fused tensor-core inference: out[n, 16] (columns 0..5 the wrench)."""
        n = feats.shape[0]
        b = tcw["b"]
        self._ck(self.lib.hydro_nn_mlp_tc(self.h.ctx, _ptr(feats), n, _ptr(self.f_mean), _ptr(self.f_istd),
                                          _ptr(tcw["image"]), _ptr(b[0]), _ptr(b[1]), _ptr(b[2]), _ptr(b[3]),
                                          _ptr(out), _ptr(tcw["err"]), self._s()))
        return out

    def _mlp(self, bufs, n_pad):
        H = self.hidden
        Ls = self.layers
        ins = [bufs["X0"], bufs["x"][0], bufs["x"][1]]
        for l in range(3):
            self.gemm(1, ins[l], Ls[l]["k"], Ls[l]["w16"], H, n_pad, H, Ls[l]["k"], y=bufs["x"][l],
                      bias=Ls[l]["b"])
        self.gemm(2, bufs["x"][2], H, bufs["w3"], OUT_PAD, n_pad, OUT_PAD, H, z=bufs["z"], bias=bufs["b3"])


class GatedPredictor:
    """Surrogate inference over a fixed number of hull states with the gate's
    rejects routed to the exact step (one exact batch over n slots; slots
    past the rejected count are switched off and cost nothing)."""

    # faces per work chunk of the exact fallback batch: eleven tiles (with
    # 650 to 1,600 of 65,536 torpedo states gated out: 4-12% faster than four
    # tiles, 1-2% faster than eight or sixteen)
    FALLBACK_CHUNK_FACES = 11 * abi.TILE_FACES

    def __init__(self, sur: Surrogate, hctx_exact: HydroContext, mesh_id: int, n: int,
                 ocean: abi.Ocean, settings: abi.Settings, tensor_cores: str = "tcgen05",
                 fallback_chunk_faces: int | None = None, second: Surrogate | None = None,
                 tau: float = float("inf"), gate_inside: bool = False, audit_stride: int = 0,
                 audit_ring: int = 256):
        """``second``: another network of the same hull; the output is then the
        mean of the two and states where they disagree by more than ``tau``
        (wrench metric) take the exact step.  ``gate_inside``: states whose
        fluid position is INSIDE take the exact step.  ``audit_stride`` > 0:
        every call also sends rows phase, phase + stride, ... that the gate
        admitted to the exact step (their output becomes exact) and records
        the network's error on them (``audit_errors``); the phase advances by
        one per call."""
        self.s = sur
        self.second = second
        self.tau = float(tau)
        self.gate_inside = gate_inside
        self.fs, self.ts = hull_scales(ocean)
        self.audit_stride = int(audit_stride)
        self.audit_k = (n + audit_stride - 1) // audit_stride if audit_stride else 0
        self.audit_ring = audit_ring
        self.audit_calls = 0
        self.h = hctx_exact
        self.lib = hctx_exact.lib
        self.n = n
        self.n_pad = (n + 63) // 64 * 64
        self.ocean = ocean
        self.settings = settings
        dev = sur.dev
        self.bufs = sur._infer_bufs(self.n_pad)
        # small chunks: only the few gated-out hulls are active per call
        self.batch = hctx_exact.batch(np.full(n, mesh_id, dtype=np.uint32),
                                      chunk_faces=fallback_chunk_faces or self.FALLBACK_CHUNK_FACES)
        self.mesh_id = mesh_id
        self.counts = torch.zeros((n + 255) // 256, dtype=torch.int32, device=dev)
        self.packed = torch.zeros(n * abi.BODY_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.pos = torch.zeros(n, dtype=torch.int32, device=dev)
        self.n_packed = torch.zeros(1, dtype=torch.int32, device=dev)
        self.exact_io = torch.zeros(n * abi.WRENCH_DTYPE.itemsize, dtype=torch.uint8, device=dev)
        self.out = torch.zeros((n, N_OUT), dtype=torch.float32, device=dev)
        self.launches = 0
        # "tcgen05": one fused kernel for the whole network; "mma": the four
        # mma.sync GEMMs of the training path
        assert tensor_cores in ("tcgen05", "mma")
        self.mode = tensor_cores
        if tensor_cores == "tcgen05":
            self.tcw = sur.tc_weights()
            self.z16 = torch.zeros((self.n_pad, 16), dtype=torch.float32, device=dev)
        if second is not None:
            assert tensor_cores == "tcgen05", "the ensemble runs on the fused tensor-core kernel"
            self.tcw2 = second.tc_weights()
            self.z16b = torch.zeros((self.n_pad, 16), dtype=torch.float32, device=dev)
        if self.audit_k:
            self.audit_idx = torch.zeros(self.audit_k, dtype=torch.int32, device=dev)
            self.audit_err = torch.full((audit_ring, self.audit_k), -1.0, dtype=torch.float32, device=dev)

    def _ck(self, st):
        _check(self.lib, self.h.ctx, st)

    def predict(self, d_bodies: torch.Tensor) -> torch.Tensor:
        """d_bodies: bytes of n hydro_body on the device, or in page-locked
        host memory, which the kernels then read in place (mesh ids are
        ignored: the exact slots use this predictor's mesh).  Returns out
        [n,6] (device)."""
        s = self.s
        st = s._s()
        n, b = self.n, self.bufs
        g = s.gate
        ctx = self.h.ctx
        if d_bodies.is_cuda:
            bodies = _ptr(d_bodies)
        else:
            bodies = C.c_void_p(abi.mapped_host_ptr(d_bodies.data_ptr()))
        self._ck(self.lib.hydro_nn_features(ctx, bodies, n, C.byref(self.ocean), _ptr(b["feats"]), st))
        self._ck(self.lib.hydro_nn_gate(ctx, _ptr(b["feats"]), n, _ptr(g["lo"]), _ptr(g["hi"]), _ptr(g["mean"]),
                                        _ptr(g["P"]), g["thr"], _ptr(b["mask"]), st))
        extra = 0
        if self.gate_inside:
            self._ck(self.lib.hydro_nn_gate_inside(ctx, bodies, n, C.byref(self.ocean), _ptr(b["mask"]), st))
            extra += 1
        if self.mode == "tcgen05":
            s.infer_tc(b["feats"], self.z16, self.tcw)
            z, ldz, mlp_launches = self.z16, 16, 1
            if self.second is not None:
                self.second.infer_tc(b["feats"], self.z16b, self.tcw2)
                self._ck(self.lib.hydro_nn_ensemble(ctx, _ptr(self.z16), _ptr(self.z16b), 16, n, self.fs, self.ts,
                                                    self.tau, _ptr(b["mask"]), st))
                extra += 2
        else:
            s.to_bf16(b["feats"], self.n_pad, N_FEAT, IN_PAD, b["X0"], s.f_mean, s.f_istd)
            s._mlp(b, self.n_pad)
            z, ldz, mlp_launches = b["z"], OUT_PAD, 5
        if self.audit_k:
            phase = self.audit_calls % self.audit_stride
            self._ck(self.lib.hydro_nn_audit_pick(ctx, _ptr(b["mask"]), n, self.audit_stride, phase, self.audit_k,
                                                  _ptr(self.audit_idx), st))
            extra += 1
        self._ck(self.lib.hydro_nn_route(ctx, bodies, _ptr(b["mask"]), n, _ptr(self.counts),
                                         _ptr(self.packed), _ptr(self.pos), _ptr(self.n_packed),
                                         _ptr(self.exact_io), st))
        self.batch.compute_device_prefix(self.packed.data_ptr(), self.n_packed.data_ptr(), self.ocean,
                                         self.settings, self.exact_io.data_ptr(), st)
        self._ck(self.lib.hydro_nn_merge(ctx, bodies, _ptr(z), ldz, _ptr(self.pos),
                                         _ptr(self.exact_io), n, _ptr(self.out), st))
        if self.audit_k:
            row = self.audit_err[self.audit_calls % self.audit_ring]
            self._ck(self.lib.hydro_nn_audit_error(ctx, bodies, _ptr(z), ldz, _ptr(self.pos), _ptr(self.exact_io),
                                                   _ptr(self.audit_idx), self.audit_k, self.fs, self.ts, _ptr(row),
                                                   st))
            self.audit_calls += 1
            extra += 1
        # features, gate (+ inside gate, second network, ensemble, audit), network, 2 route, exact step, merge
        self.launches = 1 + 1 + mlp_launches + 2 + self.batch.last_launches() + 1 + extra
        return self.out

    def admitted(self) -> np.ndarray:
        """Rows of the last call whose output is the network's (host bool array)."""
        return self.pos.cpu().numpy() < 0

    def audit_errors(self) -> np.ndarray:
        """Errors the exact step measured on the audited rows of the last
        ``audit_ring`` calls (wrench metric), one value per audited row."""
        if not self.audit_k:
            return np.zeros(0)
        e = self.audit_err.cpu().numpy().reshape(-1)
        return e[e >= 0.0]

    def rejected(self) -> int:
        return int(self.n_packed.item())

    def close(self):
        self.batch.close()


def calibrate_disagreement(pred_a: np.ndarray, pred_b: np.ndarray, exact: np.ndarray, admitted: np.ndarray,
                           ocean: abi.Ocean, target_p99: float = 0.01, max_reject: float = 0.04) -> dict:
    """Threshold on two networks' disagreement for the ensemble gate, from
    held-out states with exact labels: the smallest rejected fraction (in
    steps of 0.1%, at most ``max_reject``) whose admitted states have a 99th
    percentile error (of the mean prediction) at or below ``target_p99``;
    ``admitted`` marks the states the other gates let through."""
    fs, ts = hull_scales(ocean)
    d = np.maximum(np.linalg.norm(pred_a[:, :3] - pred_b[:, :3], axis=1) / fs,
                   np.linalg.norm(pred_a[:, 3:] - pred_b[:, 3:], axis=1) / ts)
    mean = 0.5 * (pred_a + pred_b)
    e = np.maximum(np.linalg.norm(mean[:, :3] - exact[:, :3], axis=1) / fs,
                   np.linalg.norm(mean[:, 3:] - exact[:, 3:], axis=1) / ts)
    da, ea = d[admitted], e[admitted]
    order = np.sort(da)[::-1]
    best = None
    for k in range(0, int(max_reject * 1000) + 1):
        r = k / 1000.0
        m = int(round(r * len(da)))
        tau = float(order[m - 1]) if m > 0 else float("inf")
        keep = da < tau if m > 0 else np.ones(len(da), bool)
        p99 = float(np.percentile(ea[keep], 99))
        best = {"tau": tau, "reject_frac": r, "admitted_p99": p99}
        if p99 <= target_p99:
            break
    best["target_p99"] = target_p99
    return best


def wrench_errors(pred: np.ndarray, exact: np.ndarray, ocean: abi.Ocean) -> dict:
    """Per-sample force and torque errors against the hull's scales."""
    fs, ts = hull_scales(ocean)
    ef = np.linalg.norm(pred[:, :3] - exact[:, :3], axis=1) / fs
    et = np.linalg.norm(pred[:, 3:] - exact[:, 3:], axis=1) / ts
    e = np.maximum(ef, et)
    q = lambda a, p: float(np.quantile(a, p))
    return {"force_median": q(ef, 0.5), "force_p99": q(ef, 0.99), "torque_median": q(et, 0.5),
            "torque_p99": q(et, 0.99), "wrench_mean": float(e.mean()), "wrench_median": q(e, 0.5),
            "wrench_p95": q(e, 0.95), "wrench_p99": q(e, 0.99), "wrench_max": float(e.max())}

"""Learned warm start of the moisture-form Richards solve.

A 64 -> 128 -> 128 -> 21 perceptron (SiLU hidden layers, BF16 weights and
activations, FP32 accumulation; the last layer padded to 32 outputs) proposes for
every column the number k of halvings of the step length its first substep needs
(output 0) and that substep's saturation increment per soil level (outputs 1..20).
The solver starts from dtime / 2^k (clmgb_soil_water_warm) and its own error test
accepts or halves the proposal like any substep, so the result meets the same
tolerance as the plain solve.

Training pairs come from the plain FP64 solver (clmgb_mlp_samples); training and
inference run on the GPU through the library's kernels (mma.sync linear layers,
CUDA-core weight gradients, Adam).  torch only holds the buffers.
"""
import ctypes as C
import math

import numpy as np

from . import abi, api
from ._lib import check

IN, HID, OUT, OUTP = 64, 128, 21, 32
LAYERS = [(HID, IN), (HID, HID), (OUTP, HID)]   # (out, in) per layer


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _s(stream):
    import torch
    return C.c_void_p((stream or torch.cuda.current_stream()).cuda_stream)


class WarmStartMLP:
    """Weights, optimiser state and normalisation of the warm-start network."""

    def __init__(self, handle, seed=0, device="cuda"):
        import torch
        self.h = handle
        self.torch = torch
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.wb, self.wt = [], [], [], []
        self.mw, self.vw, self.mb, self.vb = [], [], [], []
        for li, (o, i) in enumerate(LAYERS):
            w = torch.randn((o, i), generator=g, dtype=torch.float32) * math.sqrt(2.0 / i)
            if li == 2:
                w[OUT:] = 0.0
            self.w.append(w.to(device))
            self.b.append(torch.zeros(o, dtype=torch.float32, device=device))
            self.wb.append(self.w[-1].to(torch.bfloat16))
            self.wt.append(self.w[-1].t().contiguous().to(torch.bfloat16))
            for lst, shape in ((self.mw, (o, i)), (self.vw, (o, i)), (self.mb, (o,)), (self.vb, (o,))):
                lst.append(torch.zeros(shape, dtype=torch.float32, device=device))
        self.mean = torch.zeros(IN, dtype=torch.float32, device=device)
        self.istd = torch.ones(IN, dtype=torch.float32, device=device)
        self.incr_scale = 1.0
        self.margin = 0.5
        self.kmax = 6
        self.step = 0

    # ---- forward / backward through the library kernels ----
    def forward(self, X, keep=False, stream=None):
        """X: [M, 64] bf16 (normalised).  Returns Y [M, 32] fp32 (and activations)."""
        torch = self.torch
        M = X.shape[0]
        lib, h, st = self.h.lib, self.h.h, _s(stream)
        Z1 = torch.empty((M, HID), dtype=torch.float32, device=X.device)
        H1 = torch.empty((M, HID), dtype=torch.bfloat16, device=X.device)
        Z2 = torch.empty_like(Z1)
        H2 = torch.empty_like(H1)
        Y = torch.empty((M, OUTP), dtype=torch.float32, device=X.device)
        check(lib.clmgb_mlp_linear(h, M, HID, IN, _p(X), IN, _p(self.wb[0]), _p(self.b[0]), 1, _p(Z1), HID,
                                   _p(H1), HID, st), "mlp_linear 1")
        check(lib.clmgb_mlp_linear(h, M, HID, HID, _p(H1), HID, _p(self.wb[1]), _p(self.b[1]), 1, _p(Z2), HID,
                                   _p(H2), HID, st), "mlp_linear 2")
        check(lib.clmgb_mlp_linear(h, M, OUTP, HID, _p(H2), HID, _p(self.wb[2]), _p(self.b[2]), 0, _p(Y), OUTP,
                                   None, OUTP, st), "mlp_linear 3")
        if keep:
            return Y, (X, Z1, H1, Z2, H2)
        return Y

    def gradients(self, acts, dY, stream=None):
        """Backward pass: returns (dW, db) per layer (fp32)."""
        torch = self.torch
        X, Z1, H1, Z2, H2 = acts
        M = X.shape[0]
        lib, h, st = self.h.lib, self.h.h, _s(stream)
        dW = [torch.zeros_like(w) for w in self.w]
        db = [torch.zeros_like(b) for b in self.b]
        check(lib.clmgb_mlp_linear_dw(h, M, OUTP, HID, _p(dY), OUTP, _p(H2), HID, _p(dW[2]), _p(db[2]), st), "dw3")
        dH2 = torch.empty((M, HID), dtype=torch.bfloat16, device=X.device)
        check(lib.clmgb_mlp_linear(h, M, HID, OUTP, _p(dY), OUTP, _p(self.wt[2]), None, 0, None, HID, _p(dH2), HID,
                                   st), "dx3")
        dZ2 = torch.empty_like(dH2)
        check(lib.clmgb_mlp_silu_backward(h, M * HID, _p(Z2), _p(dH2), _p(dZ2), st), "silu2")
        check(lib.clmgb_mlp_linear_dw(h, M, HID, HID, _p(dZ2), HID, _p(H1), HID, _p(dW[1]), _p(db[1]), st), "dw2")
        dH1 = torch.empty_like(dH2)
        check(lib.clmgb_mlp_linear(h, M, HID, HID, _p(dZ2), HID, _p(self.wt[1]), None, 0, None, HID, _p(dH1), HID,
                                   st), "dx2")
        dZ1 = torch.empty_like(dH1)
        check(lib.clmgb_mlp_silu_backward(h, M * HID, _p(Z1), _p(dH1), _p(dZ1), st), "silu1")
        check(lib.clmgb_mlp_linear_dw(h, M, HID, IN, _p(dZ1), HID, _p(X), IN, _p(dW[0]), _p(db[0]), st), "dw1")
        return dW, db

    def loss(self, Y, T, w_dt=1.0, w_incr=1.0, stream=None):
        torch = self.torch
        M = Y.shape[0]
        l = torch.zeros(1, dtype=torch.float32, device=Y.device)
        dY = torch.empty((M, OUTP), dtype=torch.bfloat16, device=Y.device)
        check(self.h.lib.clmgb_mlp_loss(self.h.h, M, _p(Y), _p(T), float(w_dt), float(w_incr), _p(l), _p(dY),
                                        _s(stream)), "mlp_loss")
        return l, dY

    def adam(self, dW, db, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, stream=None):
        self.step += 1
        lib, h, st = self.h.lib, self.h.h, _s(stream)
        for li, (o, i) in enumerate(LAYERS):
            check(lib.clmgb_mlp_adam(h, o, i, _p(self.w[li]), _p(dW[li]), _p(self.mw[li]), _p(self.vw[li]),
                                     lr, b1, b2, eps, self.step, _p(self.wb[li]), _p(self.wt[li]), st), "adam w")
            check(lib.clmgb_mlp_adam(h, 1, o, _p(self.b[li]), _p(db[li]), _p(self.mb[li]), _p(self.vb[li]),
                                     lr, b1, b2, eps, self.step, None, None, st), "adam b")

    # ---- data ----
    def set_normalisation(self, F, T):
        """Feature mean / inverse std and the increment scale from training data."""
        torch = self.torch
        self.mean = F.mean(0).float().contiguous()
        sd = F.std(0).float()
        self.istd = torch.where(sd > 1e-6, 1.0 / sd, torch.ones_like(sd)).contiguous()
        inc = T[:, 1:OUT]
        s = float(inc.abs().mean())
        self.incr_scale = 1.0 / s if s > 0 else 1.0

    def prepare(self, F, T):
        """Normalised bf16 inputs and scaled fp32 targets."""
        X = ((F - self.mean) * self.istd).to(self.torch.bfloat16).contiguous()
        Tn = T.clone()
        Tn[:, 1:OUT] *= self.incr_scale
        return X, Tn.contiguous()

    def train(self, F, T, epochs=3, batch=4096, lr=2e-3, seed=0, log=None):
        """Adam over shuffled minibatches; returns the mean loss of each epoch."""
        torch = self.torch
        self.set_normalisation(F, T)
        X, Tn = self.prepare(F, T)
        n = X.shape[0]
        gen = torch.Generator(device=X.device).manual_seed(seed)
        hist = []
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen, device=X.device)
            tot = torch.zeros(1, dtype=torch.float32, device=X.device)
            nb = 0
            for s0 in range(0, n - batch + 1, batch):
                idx = perm[s0:s0 + batch]
                xb, tb = X[idx].contiguous(), Tn[idx].contiguous()
                Y, acts = self.forward(xb, keep=True)
                l, dY = self.loss(Y, tb)
                dW, db = self.gradients(acts, dY)
                self.adam(dW, db, lr=lr * (0.8 ** ep))
                tot += l
                nb += 1
            hist.append(float(tot) / max(nb, 1))
            if log:
                log("epoch %d loss %.4f" % (ep, hist[-1]))
        return hist

    # ---- use in the solver ----
    def features(self, state, dtime, cfg=None, out=None, stream=None):
        """The normalised BF16 feature rows [nc x 64] of the state at the start of soil_water."""
        cfg = cfg or abi.SwmConfig.clm5_default()
        X = out if out is not None else self.torch.empty((state.nc, IN), dtype=self.torch.bfloat16, device="cuda")
        b, fw = state.bounds(), state.soilwater_fields()
        check(self.h.lib.clmgb_mlp_features(self.h.h, C.byref(b), C.byref(fw), C.byref(cfg), float(dtime),
                                            _p(self.mean), _p(self.istd), _p(X), _s(stream)), "mlp_features")
        return X

    def propose_first_dt(self, state, dtime, cfg=None, out=None, stream=None):
        """dt_first [nc] (float64) for the state at the start of soil_water."""
        torch = self.torch
        nc = state.nc
        X = self.features(state, dtime, cfg, stream=stream)
        Y = self.forward(X, stream=stream)
        dt = out if out is not None else torch.empty(nc, dtype=torch.float64, device="cuda")
        check(self.h.lib.clmgb_mlp_first_dt(self.h.h, nc, _p(Y), float(dtime), float(self.margin), int(self.kmax),
                                            _p(dt), _s(stream)), "mlp_first_dt")
        return dt

    def state_dict(self):
        d = {"w%d" % i: w.cpu().numpy() for i, w in enumerate(self.w)}
        d.update({"b%d" % i: b.cpu().numpy() for i, b in enumerate(self.b)})
        d.update({"mean": self.mean.cpu().numpy(), "istd": self.istd.cpu().numpy(),
                  "incr_scale": np.array(self.incr_scale), "margin": np.array(self.margin),
                  "kmax": np.array(self.kmax)})
        return d

    def load_state_dict(self, d):
        torch = self.torch
        for i in range(3):
            self.w[i] = torch.from_numpy(np.asarray(d["w%d" % i], dtype=np.float32)).cuda()
            self.b[i] = torch.from_numpy(np.asarray(d["b%d" % i], dtype=np.float32)).cuda()
            self.wb[i] = self.w[i].to(torch.bfloat16)
            self.wt[i] = self.w[i].t().contiguous().to(torch.bfloat16)
        self.mean = torch.from_numpy(np.asarray(d["mean"], dtype=np.float32)).cuda()
        self.istd = torch.from_numpy(np.asarray(d["istd"], dtype=np.float32)).cuda()
        self.incr_scale = float(d["incr_scale"])
        self.margin = float(d["margin"])
        self.kmax = int(d["kmax"])


def soil_water_warm(handle, state, dtime, dt_first, cfg=None, col_status=None, stream=None):
    """soil_water! with the proposed first substep per column (clmgb_soil_water_warm)."""
    cfg = cfg or abi.SwmConfig.clm5_default()
    check(handle.lib.clmgb_soil_water_warm(handle.h, C.byref(state.bounds()), C.byref(state.soilwater_fields()),
                                           C.byref(cfg), float(dtime), _p(dt_first), _p(col_status), _s(stream)),
          "soil_water_warm")


def generate_samples(handle, state, G, I, nsteps, dtime, per_column=1, capacity=None, cfg=None,
                     snow_method=abi.SNOW_JORDAN1991, record_every=1):
    """Runs nsteps plain steps (forcing, soil_temperature!, fractions, and the plain
    Richards solve, which records pairs at every `record_every`-th step, so the pairs
    cover the states of a long trajectory) and returns (features [n, 64], targets [n, 32])."""
    import torch
    cfg = cfg or abi.SwmConfig.clm5_default()
    every = max(1, int(record_every))
    nrec = (nsteps + every - 1) // every
    cap = capacity or state.nc * nrec * per_column
    F = torch.empty((cap, IN), dtype=torch.float32, device="cuda")
    T = torch.empty((cap, OUTP), dtype=torch.float32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    for t in range(nsteps):
        api.synth_forcing(handle, state, G[t], I[t])
        api.soil_temperature(handle, state, dtime, snow_method)
        api.set_soil_water_fractions(handle, state)
        if t % every:
            api.soil_water(handle, state, dtime, cfg)
            continue
        check(handle.lib.clmgb_mlp_samples(handle.h, C.byref(state.bounds()), C.byref(state.soilwater_fields()),
                                           C.byref(cfg), float(dtime), int(per_column), _p(F), _p(T), _p(cnt), cap,
                                           None, _s(None)), "mlp_samples")
    n = min(int(cnt.item()), cap)
    return F[:n], T[:n]

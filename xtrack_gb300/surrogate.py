"""Learned screening of dynamic-aperture scans.

A multilayer perceptron (default: 4 hidden layers of width 256, GELU in
its tanh form) predicts, from a particle's normalised initial coordinates
and its seed's multipole-error summary, the probability that it survives
the turn budget and, if lost, its normalised log loss turn. It is trained on the
``state`` / ``at_turn`` maps that batched tracking produces, entirely with
the library's own kernels: BF16 tensor-core contractions with FP32
accumulation for forward and backward passes, a fixed-order bias-gradient
reduction and an Adam step on FP32 master weights (include/xtrack_gb300.h,
``xtg_mlp_*``). Torch only holds the device memory.

``screen`` then tracks only the particles the network is unsure about
(P(survive) between two thresholds) plus a random audit fraction and takes
the network's answer for the rest; ``screen_rays`` does the same per ray
of a DA scan, tracking the band from the first uncertain amplitude to the
first confidently lost one. A DA scan adds ``sentinels`` (every k-th
amplitude of each ray) to that band and, in a second pass, tracks the
``bracket`` between the last surviving and the first lost tracked
amplitude of each ray (``scan.screened_da_scan``). Plain tracking of every
particle stays the reference the screened result is judged against (DA
error in beam sigma, misclassification rate on the audit).

No reference counterpart: xtrack has no learned component.
"""
import ctypes
import math

import numpy as np
import torch

from . import _abi

N_SEED_FEATURES = 32
N_COORD_FEATURES = 6
N_DA_FEATURES = N_COORD_FEATURES + 8


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _pad8(n):
    return (int(n) + 7) // 8 * 8


N_OUT = 2


class SurvivalMLP:
    """MLP n_in -> width (x depth, tanh-form GELU) -> 2 outputs, BF16
    weights and activations, FP32 accumulation, Adam on FP32 master
    weights.

    The input and output widths are padded to multiples of 8 (``dims``), so
    that every operand row is a multiple of 16 bytes and the contractions
    stage it by TMA; the padded input columns are zero, the padded output
    rows of the last weight matrix are zero and receive zero gradients, so
    the padding changes no result."""

    def __init__(self, n_in=N_COORD_FEATURES + N_SEED_FEATURES, width=256, depth=4, seed=0,
                 device="cuda", w_turn=0.5):
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise RuntimeError("SurvivalMLP runs on a CUDA device only")
        self._lib = _abi.load_library()
        self.n_in = int(n_in)
        self.dims = [_pad8(n_in)] + [width] * depth + [_pad8(N_OUT)]
        self.w_turn = float(w_turn)
        g = torch.Generator().manual_seed(seed)
        self.W, self.b = [], []
        real = [self.n_in] + [width] * depth + [N_OUT]
        for l, (k_in, k_out) in enumerate(zip(self.dims[:-1], self.dims[1:])):
            std = math.sqrt(2.0 / real[l])
            w = torch.zeros(k_out, k_in, dtype=torch.float64)
            w[:real[l + 1], :real[l]] = torch.randn(real[l + 1], real[l], generator=g,
                                                    dtype=torch.float64) * std
            self.W.append(w.float().to(self.device))
            self.b.append(torch.zeros(k_out, dtype=torch.float32, device=self.device))
        self.W16 = [w.to(torch.bfloat16) for w in self.W]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.gW = [torch.zeros_like(w) for w in self.W]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self.step_count = 0
        self.x_mean = torch.zeros(self.dims[0], dtype=torch.float32, device=self.device)
        self.x_std = torch.ones(self.dims[0], dtype=torch.float32, device=self.device)
        self._acts = None

    # ------------------------------------------------------------------
    @property
    def n_layers(self):
        return len(self.W)

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _padded(self, X):
        X = torch.as_tensor(X, dtype=torch.float32, device=self.device)
        if X.shape[1] not in (self.n_in, self.dims[0]):
            raise ValueError(f"expected {self.n_in} features, got {X.shape[1]}")
        if X.shape[1] < self.dims[0]:
            X = torch.nn.functional.pad(X, (0, self.dims[0] - X.shape[1]))
        return X

    def set_normalisation(self, X):
        X = self._padded(X)
        self.x_mean = X.mean(0)
        self.x_std = X.std(0).clamp_min(1e-12)

    def prepare_input(self, X):
        """Normalised BF16 copy of the features (fp32 [B, n_in]), padded
        with zero columns to ``dims[0]``."""
        X = self._padded(X)
        Xn = ((X - self.x_mean) / self.x_std).contiguous()
        X16 = torch.empty(Xn.shape, dtype=torch.bfloat16, device=self.device)
        _abi.check_mlp(self._lib.xtg_mlp_to_bf16(_ptr(Xn), Xn.numel(), _ptr(X16), self._stream()),
                       self._lib)
        return X16

    def forward(self, X16, keep=False):
        """Outputs fp32 [B, dims[-1]] for BF16 input [B, dims[0]]: column 0
        is the logit of P(survive), column 1 the normalised log loss turn,
        the others are padding (zero). Keeps the activations for
        ``backward`` when ``keep``; otherwise the hidden layers store only
        their BF16 activations."""
        B = X16.shape[0]
        st = self._stream()
        acts = [(None, X16)]
        y = X16
        out = None
        for l in range(self.n_layers):
            k_in, k_out = self.dims[l], self.dims[l + 1]
            last = l == self.n_layers - 1
            Z = torch.empty(B, k_out, dtype=torch.float32, device=self.device) if (keep or last) else None
            Y = None if last else torch.empty(B, k_out, dtype=torch.bfloat16, device=self.device)
            _abi.check_mlp(self._lib.xtg_mlp_gemm(
                _ptr(y), k_in, 1, _ptr(self.W16[l]), k_in, 1, B, k_out, k_in, _ptr(self.b[l]),
                _abi.MLP_ACT_NONE if last else _abi.MLP_ACT_GELU, _ptr(Z), k_out,
                _ptr(Y), k_out, None, 0, 0, st), self._lib)
            acts.append((Z, Y))
            y = Y
            out = Z
        self._acts = acts if keep else None
        return out

    def loss_and_grad(self, out, survive, logturn):
        B = out.shape[0]
        st = self._stream()
        ld = out.shape[1]
        dout = torch.zeros(B, ld, dtype=torch.float32, device=self.device)
        dout16 = torch.zeros(B, ld, dtype=torch.bfloat16, device=self.device)
        loss = torch.empty(B, dtype=torch.float32, device=self.device)
        _abi.check_mlp(self._lib.xtg_mlp_loss(_ptr(out), ld, _ptr(survive), _ptr(logturn), B,
                                              self.w_turn, _ptr(dout), _ptr(dout16), _ptr(loss),
                                              st), self._lib)
        return loss, dout, dout16

    def backward(self, dout, dout16):
        """Fills self.gW / self.gb from the kept activations."""
        if self._acts is None:
            raise RuntimeError("forward(keep=True) must precede backward")
        st = self._stream()
        B = dout.shape[0]
        dZ, dZ16 = dout, dout16
        for l in range(self.n_layers - 1, -1, -1):
            k_in, k_out = self.dims[l], self.dims[l + 1]
            y_prev = self._acts[l][1]                      # bf16 [B, k_in]
            # dW[n, k] = sum_b dZ[b, n] y_prev[b, k]
            _abi.check_mlp(self._lib.xtg_mlp_gemm(
                _ptr(dZ16), 1, k_out, _ptr(y_prev), 1, k_in, k_out, k_in, B, None,
                _abi.MLP_ACT_NONE, None, 0, None, 0, _ptr(self.gW[l]), k_in, 0, st), self._lib)
            _abi.check_mlp(self._lib.xtg_mlp_colsum(_ptr(dZ), B, k_out, k_out, _ptr(self.gb[l]),
                                                    0, st), self._lib)
            if l == 0:
                break
            # dY_prev[b, k] = sum_n dZ[b, n] W[n, k]
            dY = torch.empty(B, k_in, dtype=torch.float32, device=self.device)
            _abi.check_mlp(self._lib.xtg_mlp_gemm(
                _ptr(dZ16), k_out, 1, _ptr(self.W16[l]), 1, k_in, B, k_in, k_out, None,
                _abi.MLP_ACT_NONE, None, 0, None, 0, _ptr(dY), k_in, 0, st), self._lib)
            Z_prev = self._acts[l][0]
            dZ = torch.empty(B, k_in, dtype=torch.float32, device=self.device)
            dZ16 = torch.empty(B, k_in, dtype=torch.bfloat16, device=self.device)
            _abi.check_mlp(self._lib.xtg_mlp_act_backward(_ptr(dY), _ptr(Z_prev), dY.numel(),
                                                          _abi.MLP_ACT_GELU, _ptr(dZ), _ptr(dZ16),
                                                          st), self._lib)

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step_count += 1
        st = self._stream()
        for l in range(self.n_layers):
            _abi.check_mlp(self._lib.xtg_mlp_adam(
                _ptr(self.W[l]), _ptr(self.W16[l]), _ptr(self.gW[l]), _ptr(self.mW[l]),
                _ptr(self.vW[l]), self.W[l].numel(), lr, beta1, beta2, eps, weight_decay,
                self.step_count, st), self._lib)
            _abi.check_mlp(self._lib.xtg_mlp_adam(
                _ptr(self.b[l]), None, _ptr(self.gb[l]), _ptr(self.mb[l]), _ptr(self.vb[l]),
                self.b[l].numel(), lr, beta1, beta2, eps, 0.0, self.step_count, st), self._lib)

    # ------------------------------------------------------------------
    def fit(self, X, survive, logturn, epochs=10, batch=4096, lr=1e-3, seed=0, lr_final=None,
            weight_decay=0.0):
        """Adam training on (X, survive, logturn); returns the mean loss of
        each epoch. ``lr`` decays linearly to ``lr_final`` (default lr/10)."""
        X = torch.as_tensor(X, dtype=torch.float32, device=self.device)
        s = torch.as_tensor(survive, dtype=torch.float32, device=self.device).contiguous()
        t = torch.as_tensor(logturn, dtype=torch.float32, device=self.device).contiguous()
        self.set_normalisation(X)
        X16 = self.prepare_input(X)
        n = X16.shape[0]
        g = torch.Generator(device="cpu").manual_seed(seed)
        hist = []
        steps_total = epochs * max(1, (n + batch - 1) // batch)
        lr_final = lr / 10 if lr_final is None else lr_final
        k = 0
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.device)
            tot = torch.zeros((), dtype=torch.float64, device=self.device)
            for i0 in range(0, n, batch):
                idx = perm[i0:i0 + batch]
                xb = X16.index_select(0, idx).contiguous()
                out = self.forward(xb, keep=True)
                loss, dout, dout16 = self.loss_and_grad(out, s.index_select(0, idx).contiguous(),
                                                        t.index_select(0, idx).contiguous())
                self.backward(dout, dout16)
                cur = lr + (lr_final - lr) * k / max(1, steps_total - 1)
                self.adam_step(lr=cur, weight_decay=weight_decay)
                tot += loss.double().sum()
                k += 1
            hist.append(float(tot.item()) / n)
        return hist

    def predict(self, X, batch=65536):
        """(P(survive), normalised log loss turn) as numpy arrays."""
        X16 = self.prepare_input(X)
        ps, ts = [], []
        for i0 in range(0, X16.shape[0], batch):
            out = self.forward(X16[i0:i0 + batch].contiguous())
            ps.append(torch.sigmoid(out[:, 0]).cpu().numpy())
            ts.append(out[:, 1].cpu().numpy())
        _abi.check_mlp(self._lib.xtg_mlp_device_status(), self._lib)
        return np.concatenate(ps), np.concatenate(ts)


# ----------------------------------------------------------------------
# features and targets
# ----------------------------------------------------------------------
_FAMILIES = ("Bend", "Quadrupole", "Sextupole", "Multipole")
_MAIN_ORDER = {"Bend": 0, "Quadrupole": 1, "Sextupole": 2}
_R_REF = 0.017


def seed_features(line, r_ref=_R_REF):
    """32 numbers that summarise a seed's multipole errors, orders 0..10.
    Each knl_rel / ksl_rel entry of order n of a magnet with main order m
    is turned into the relative field error at radius r_ref,
    b_n = knl_rel[n] * m! / n! * r_ref^(n - m) (a_n from ksl_rel), in units
    of 1e-4. Per magnet family (bends, quadrupoles, sextupoles, thin
    multipoles): the family mean of b_0..b_3, of a_0 and a_1, and the RMS
    over orders of the family means of b_4..b_10 and of a_2..a_10. Means,
    not RMS over magnets: the RMS of independent errors is the same for
    every seed, the mean (the systematic part the magnets share) is not."""
    acc = {(f, n, s): [] for f in _FAMILIES for n in range(11) for s in (0, 1)}
    for name in line.element_names:
        e = line.element_dict[name]
        fam = type(e).__name__
        if fam not in _FAMILIES:
            continue
        m = _MAIN_ORDER.get(fam, int(getattr(e, "main_order", 0) or 0))
        for s, arr in ((0, getattr(e, "knl_rel", None)), (1, getattr(e, "ksl_rel", None))):
            arr = np.zeros(1) if arr is None else np.asarray(arr, dtype=np.float64)
            for n in range(11):
                v = arr[n] if n < len(arr) else 0.0
                acc[(fam, n, s)].append(v * math.factorial(m) / math.factorial(n) * r_ref ** (n - m) * 1e4)
    out = []
    for f in _FAMILIES:
        mean = {(n, s): (float(np.mean(acc[(f, n, s)])) if acc[(f, n, s)] else 0.0)
                for n in range(11) for s in (0, 1)}
        out += [mean[(n, 0)] for n in range(4)] + [mean[(0, 1)], mean[(1, 1)]]
        out.append(math.sqrt(np.mean([mean[(n, 0)] ** 2 for n in range(4, 11)])))
        out.append(math.sqrt(np.mean([mean[(n, 1)] ** 2 for n in range(2, 11)])))
    return np.asarray(out, dtype=np.float64)


def coord_features(r, theta, delta, delta_scale=2.7e-4):
    """Six normalised initial-condition features of a polar-grid particle."""
    r = np.asarray(r, dtype=np.float64)
    theta = np.asarray(theta, dtype=np.float64)
    d = np.broadcast_to(np.asarray(delta, dtype=np.float64), r.shape)
    return np.stack([r * np.cos(theta), r * np.sin(theta), r, theta, d / delta_scale,
                     (r * np.cos(theta)) ** 2 + 0.5 * (r * np.sin(theta)) ** 2], axis=1)


def da_features(scan):
    """Features of each particle of a DA scan (``scan.Scan``): its
    coordinates (``coord_features``), its seed's linear tunes and
    closed-orbit extremes (mm), its ray's linear aperture (sigma) and the
    ratio of its amplitude to it. N_DA_FEATURES columns."""
    li = scan.lattice_index
    rl = scan.ray_r_lin()
    return np.concatenate([coord_features(scan.r, scan.theta, scan.deltas[scan.delta_index]),
                           scan.tunes[li][:, :2], 1e3 * scan.co_extremes[li], rl[:, None],
                           (scan.r / np.maximum(rl, 1e-9))[:, None]], axis=1)


def targets(state, at_turn, num_turns):
    """(survive, normalised log loss turn) from a tracking result."""
    state = np.asarray(state)
    at_turn = np.asarray(at_turn, dtype=np.float64)
    survive = ((state > 0) | (at_turn >= num_turns)).astype(np.float32)
    logturn = (np.log10(at_turn + 1.0) / math.log10(num_turns + 1.0)).astype(np.float32)
    return survive, logturn


def screen(p_survive, lo=0.05, hi=0.95, audit=0.02, seed=0):
    """Boolean masks (track, audit): particles with lo < P < hi are tracked;
    an extra random ``audit`` fraction of the others is tracked too."""
    p = np.asarray(p_survive)
    unsure = (p > lo) & (p < hi)
    rng = np.random.default_rng(seed)
    aud = (~unsure) & (rng.random(p.shape) < audit)
    return unsure | aud, aud


def screen_rays(p_survive, r, ray_id, lo=0.05, hi=0.95, audit=0.02, seed=0):
    """Boolean masks (track, audit) for a DA scan on rays: on each ray the
    particles from the first amplitude the network is unsure about
    (P < hi) up to the first amplitude it calls lost (P <= lo) are
    tracked; below that band the particles are taken to survive, above it
    to be lost (they cannot change the ray's DA, the smallest lost
    amplitude), plus a random ``audit`` fraction of the rest."""
    p = np.asarray(p_survive)
    r = np.asarray(r)
    ray_id = np.asarray(ray_id)
    track = np.zeros(p.shape, dtype=bool)
    order = np.lexsort((r, ray_id))
    rid = ray_id[order]
    starts = np.flatnonzero(np.r_[True, rid[1:] != rid[:-1]])
    ends = np.r_[starts[1:], len(order)]
    for a, b in zip(starts, ends):
        idx = order[a:b]
        pr = p[idx]
        unsure = np.flatnonzero(pr < hi)
        if unsure.size == 0:
            continue
        first = unsure[0]
        lost = np.flatnonzero(pr[first:] <= lo)
        last = first + lost[0] if lost.size else len(idx) - 1
        track[idx[first:last + 1]] = True
    rng = np.random.default_rng(seed)
    aud = (~track) & (rng.random(p.shape) < audit)
    return track | aud, aud


def ray_outcome(p_survive, r, ray_id, tracked_mask, tracked_survive, hi=0.95, audit_mask=None):
    """Survival map of a ray-screened scan: tracked particles their tracked
    outcome; untracked ones below their ray's tracked band survive, above
    it are lost (audited particles are tracked but not part of the band)."""
    p = np.asarray(p_survive)
    r = np.asarray(r)
    ray_id = np.asarray(ray_id)
    out = np.zeros(p.shape, dtype=bool)
    out[tracked_mask] = np.asarray(tracked_survive, dtype=bool)
    in_band = tracked_mask if audit_mask is None else tracked_mask & ~np.asarray(audit_mask)
    for rid in np.unique(ray_id):
        on = ray_id == rid
        band = on & in_band
        untracked = on & ~tracked_mask
        if band.any():
            r_band_lo = r[band].min()
            out[untracked] = r[untracked] < r_band_lo
        else:
            out[untracked] = p[untracked] >= hi
    return out


def _rays(r, ray_id):
    """Particle indices sorted by (ray, amplitude) and the [start, end) of
    each ray in that order."""
    order = np.lexsort((np.asarray(r), np.asarray(ray_id)))
    rid = np.asarray(ray_id)[order]
    starts = np.flatnonzero(np.r_[True, rid[1:] != rid[:-1]]) if len(rid) else np.zeros(0, np.int64)
    ends = np.r_[starts[1:], len(order)]
    return order, starts, ends


def sentinels(r, ray_id, stride):
    """Mask of every ``stride``-th amplitude of each ray, counted from the
    smallest, plus the largest."""
    mask = np.zeros(len(r), dtype=bool)
    order, starts, ends = _rays(r, ray_id)
    for a, b in zip(starts, ends):
        idx = order[a:b]
        mask[idx[::stride]] = True
        mask[idx[-1]] = True
    return mask


def thin(mask, r, ray_id, stride):
    """Every ``stride``-th particle of ``mask`` on each ray, counted by
    amplitude from the smallest, plus the ray's largest masked one."""
    mask = np.asarray(mask, dtype=bool)
    sel = np.flatnonzero(mask)
    out = np.zeros(len(mask), dtype=bool)
    out[sel[sentinels(np.asarray(r)[sel], np.asarray(ray_id)[sel], stride)]] = True
    return out


def bracket(r, ray_id, tracked_mask, survive):
    """Mask of the untracked particles of each ray between the largest
    tracked survivor below the ray's smallest tracked loss and that loss:
    the amplitudes where the ray's DA can still lie. ``survive`` is read
    where ``tracked_mask`` is set."""
    tracked_mask = np.asarray(tracked_mask, dtype=bool)
    survive = np.asarray(survive, dtype=bool)
    mask = np.zeros(len(r), dtype=bool)
    order, starts, ends = _rays(r, ray_id)
    for a, b in zip(starts, ends):
        idx = order[a:b]
        t = np.flatnonzero(tracked_mask[idx])
        lost = t[~survive[idx[t]]]
        if lost.size == 0:
            continue
        first = lost[0]
        below = t[t < first]
        lo = below[-1] + 1 if below.size else 0
        mask[idx[lo:first]] = True
    return mask


def ray_survival(r, ray_id, tracked_mask, survive):
    """Survival map of a sentinel/bracket scan: tracked particles keep their
    outcome; an untracked particle survives if it lies below its ray's
    smallest tracked loss (so the map's DA per ray is that loss)."""
    tracked_mask = np.asarray(tracked_mask, dtype=bool)
    out = np.where(tracked_mask, np.asarray(survive, dtype=bool), False)
    order, starts, ends = _rays(r, ray_id)
    r = np.asarray(r)
    for a, b in zip(starts, ends):
        idx = order[a:b]
        lost = idx[tracked_mask[idx] & ~out[idx]]
        r_loss = r[lost].min() if lost.size else np.inf
        un = idx[~tracked_mask[idx]]
        out[un] = r[un] < r_loss
    return out


def screened_outcome(p_survive, tracked_mask, tracked_survive, hi=0.95):
    """Survival map of a screened scan: the tracked particles' outcome where
    tracked, else the network's (P >= hi: survives)."""
    out = np.asarray(p_survive) >= hi
    out = out.copy()
    out[tracked_mask] = np.asarray(tracked_survive, dtype=bool)
    return out

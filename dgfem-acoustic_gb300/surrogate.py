"""Learned spectral surrogate of the batched DG ensemble.

Maps the parameters of one 2-D LEE instance -- monopole position (x, y),
frequency f, mean-flow Mach number M and angle th, element order p -- to the
log power spectral density of the pressure at the ensemble's four observers
(128 bins each), with a fully connected network (6 -> 4 x 256 GELU -> 512,
BF16 weights, FP32 accumulation) that is trained and evaluated on the GPU by
the project's own kernels (gpu.Network, csrc/mlp.cu).

The reference has no counterpart: it answers every query with a DG run. DG
stays the measure of the network's error and its fallback here: the training and test targets come
from batched DG runs, and a query whose estimated spectral error exceeds the
bound is re-run through DG. The error estimate is the spread of independently
trained networks around their mean (four by default), scaled so that it
covers the true error of 95 % of a calibration split.

Targets: the last power-of-two samples of the observer pressure trace of
STEPS RK4 steps (the settled part: the first samples hold the wave-front
arrival), Hann-tapered, power-normalised and zero-padded eightfold, go
through the project's restatement of the reference's PSD_spec (host.spectra:
mean removed, one-sided periodogram, src/fft.cpp:183-227); the linear power
is averaged over 128 bins of the source-frequency axis nu = f'/f in
[0, NU_MAX) (bin means of the piecewise-linear PSD; bin_frequencies maps
them back to Hz) and expressed in dB re (20 uPa)^2, floored DYN_RANGE_DB
below each observer's peak bin. The taper replaces the rectangular window's
leakage pattern by a compact main lobe; the relative axis keeps the tone at
nu = 1 for every query, so that the network learns its level and lobe shape
rather than a peak sliding across fixed bins; the padding and the bin
integrals make each bin a smooth function of the tone's position between
FFT lines (without them the tone's bin level moves by up to 1.4 dB with f
times the record length, faster than the parameter sampling resolves).
Instances use one fixed jittered GRID x GRID mesh per order, so the spectrum
is a function of the six parameters alone.
"""
import importlib
import math
import time

import numpy as np

WIDTHS = [6, 256, 256, 256, 256, 512]
N_OBS, N_BINS = 4, 128
NU_MAX = 4.0  # bins span [0, NU_MAX) source-frequency multiples
DYN_RANGE_DB = 30.0
ZERO_PAD = 8  # FFT length / analysed samples
STEPS = 3000
GRID = 25
MESH_SEEDS = {2: 502, 3: 503, 4: 504}


def _pkg():
    return importlib.import_module(__name__.rsplit(".", 1)[0])


def draw_params(n, seed):
    """[n][6] rows (x, y, f, M, th, p) with the ensemble's distributions."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 6))
    out[:, 0:2] = rng.uniform(-4, 4, (n, 2))
    out[:, 2] = rng.uniform(20, 400, n)
    out[:, 3] = rng.uniform(0, 0.3, n)
    out[:, 4] = rng.uniform(0, 2 * np.pi, n)
    out[:, 5] = rng.integers(2, 5, n)
    return out


def features(params):
    """Network inputs: position / 4, centred frequency, the mean-flow vector
    (M cos th, M sin th) / 0.3 (continuous in the angle), p - 3."""
    P = np.asarray(params, dtype=np.float64).reshape(-1, 6)
    x = np.empty((P.shape[0], 6), dtype=np.float32)
    x[:, 0] = P[:, 0] / 4
    x[:, 1] = P[:, 1] / 4
    x[:, 2] = (P[:, 2] - 210.0) / 190.0
    x[:, 3] = P[:, 3] * np.cos(P[:, 4]) / 0.3
    x[:, 4] = P[:, 3] * np.sin(P[:, 4]) / 0.3
    x[:, 5] = P[:, 5] - 3.0
    return x


def bin_frequencies(f):
    """Centre frequencies (Hz) of the 128 bins for source frequency f."""
    return (np.arange(N_BINS) + 0.5) * (NU_MAX / N_BINS) * f


def log_psd_bins(trace, dt, f):
    """128-bin log-PSD (dB re (20 uPa)^2) of one pressure trace on the
    source-frequency axis nu = f'/f in [0, NU_MAX): the last power-of-two
    samples n (the settled part of the run), their Hann-weighted mean
    removed, Hann-tapered, power-normalised and zero-padded to ZERO_PAD * n
    samples, through the PSD_spec restatement (rescaled to the unpadded
    segment's PSD level); each bin is the mean over its frequency interval
    of the piecewise-linear PSD between the FFT lines."""
    tr = np.asarray(trace, dtype=np.float64)
    n = 1
    while n * 2 <= len(tr):
        n *= 2
    seg = tr[len(tr) - n:]
    w = 0.5 * (1.0 - np.cos(2 * np.pi * np.arange(n) / (n - 1)))
    x = np.zeros(ZERO_PAD * n)
    # a zero-mean padded record: PSD_spec's own mean removal changes nothing
    x[:n] = (seg - np.sum(seg * w) / np.sum(w)) * w / math.sqrt(np.mean(w * w))
    _, psd = _pkg().host.spectra(x.astype(np.float32), dt)
    m = ZERO_PAD * n
    fl, P = psd[:, 0], psd[:, 1] * (ZERO_PAD * ZERO_PAD * (n - 1) / (m - 1))
    edges = np.arange(N_BINS + 1) * (NU_MAX / N_BINS) * f
    # exact integrals of the piecewise-linear PSD up to each bin edge
    C = np.concatenate([[0.0], np.cumsum(0.5 * (P[1:] + P[:-1]) * np.diff(fl))])
    i = np.clip(np.searchsorted(fl, edges, side="right") - 1, 0, len(fl) - 2)
    xe = np.clip(edges, fl[0], fl[-1])
    pe = P[i] + (xe - fl[i]) / (fl[i + 1] - fl[i]) * (P[i + 1] - P[i])
    Ce = C[i] + (xe - fl[i]) * 0.5 * (P[i] + pe)
    out = np.diff(Ce) / np.diff(edges)
    peak = out.max()
    out = np.maximum(out, peak * 10 ** (-DYN_RANGE_DB / 10) if peak > 0 else 1e-30)
    return 10 * np.log10(out / (2e-5) ** 2)


_MESH_CACHE = {}


def _meshes(grid):
    if grid not in _MESH_CACHE:
        ens = _pkg().ensemble
        _MESH_CACHE[grid] = {p: ens.square_mesh(grid, p, MESH_SEEDS[p]) for p in (2, 3, 4)}
    return _MESH_CACHE[grid]


def dg_spectra(params, chunk=2000, steps=STEPS, grid=GRID, precision=None, progress=None):
    """DG targets for parameter rows: [n][N_OBS][N_BINS] log-PSD, and the
    seconds spent in the batched DG runs (setup excluded)."""
    pkg = _pkg()
    ens, gpu = pkg.ensemble, pkg.gpu
    precision = gpu.DG_FP32 if precision is None else precision
    meshes = _meshes(grid)
    P = np.asarray(params, dtype=np.float64).reshape(-1, 6)
    out = np.zeros((P.shape[0], N_OBS, N_BINS))
    dg_s = 0.0
    for c0 in range(0, P.shape[0], chunk):
        rows = P[c0:c0 + chunk]
        insts = [ens.instance(meshes[int(r[5])], int(r[5]), r[0], r[1], r[2], r[3], r[4]) for r in rows]
        B = ens.make_batch(insts, precision, steps)
        traces = [np.zeros((steps, N_OBS)) for _ in insts]
        t0 = time.perf_counter()
        done, seg = 0, 500
        while done < steps:
            n = min(seg, steps - done)
            obs = B.run(n)
            for k, o in enumerate(obs):
                traces[k][done:done + n] = o[:, :, 0]
            done += n
        dg_s += time.perf_counter() - t0
        B.close()
        for k, i in enumerate(insts):
            for o in range(N_OBS):
                out[c0 + k, o] = log_psd_bins(traces[k][:, o], i["dt"], i["src"][5])
        if progress:
            progress(c0 + len(rows), P.shape[0])
    return out, dg_s


def rms_db(a, b):
    """Per-query RMS over all observers and bins of the dB difference."""
    d = np.asarray(a, dtype=np.float64).reshape(len(a), -1) - np.asarray(b, dtype=np.float64).reshape(len(b), -1)
    return np.sqrt(np.mean(d * d, axis=1))


class Surrogate:
    """Independently trained networks (four by default), target normalisation
    and the calibrated error estimate (the members' spread)."""

    def __init__(self, params_list, mu, sigma, scale=1.0, grid=GRID, steps=STEPS, device=0):
        self.mu = np.asarray(mu, dtype=np.float32)
        self.sigma = float(sigma)
        self.scale = float(scale)
        self.grid, self.steps = int(grid), int(steps)  # the DG runs the targets came from
        self.nets = []
        for p in params_list:
            net = _pkg().gpu.Network(WIDTHS, device=device)
            net.set_params(p)
            self.nets.append(net)

    @classmethod
    def fit(cls, params, targets, n_models=4, steps=10000, batch=256, lr=4e-3, lr_final=2e-5, seed=0, grid=GRID,
            dg_steps=STEPS, weight_decay=0.1, device=0):
        x = features(params)
        y = np.asarray(targets, dtype=np.float64).reshape(len(x), -1)
        mu = y.mean(axis=0)
        sigma = float((y - mu).std())
        t = ((y - mu) / sigma).astype(np.float32)
        rng = np.random.default_rng(seed)
        plist, losses = [], []
        for m in range(n_models):
            net = _pkg().gpu.Network(WIDTHS, device=device)
            net.set_params(_init(WIDTHS, int(rng.integers(1 << 30))))
            net.set_data(x, t)
            losses.append(net.train(steps, batch, lr, lr_final, seed=int(rng.integers(1 << 62)),
                                    weight_decay=weight_decay))
            plist.append(net.get_params())
            net.close()
        s = cls(plist, mu, sigma, grid=grid, steps=dg_steps, device=device)
        s.train_losses = losses
        return s

    def predict(self, params):
        """Mean prediction [n][N_OBS][N_BINS] (dB) and the estimated RMS error
        per query (dB)."""
        x = features(params)
        ys = [net.forward(x).astype(np.float64) * self.sigma + self.mu for net in self.nets]
        mean = np.mean(ys, axis=0)
        if len(ys) > 1:
            # spread of the members around their mean (RMS over outputs)
            est = self.scale * np.sqrt(np.mean([rms_db(y, mean) ** 2 for y in ys], axis=0) * len(ys) / (len(ys) - 1))
        else:
            est = np.zeros(len(x))
        return mean.reshape(-1, N_OBS, N_BINS), est

    def calibrate(self, params, targets, coverage=0.95):
        """Scale the disagreement so that it bounds the true error of the
        given fraction of these (held-out) queries."""
        self.scale = 1.0
        mean, est = self.predict(params)
        err = rms_db(mean, targets)
        ratio = err / np.maximum(est, 1e-12)
        self.scale = float(np.quantile(ratio, coverage))
        return self.scale

    def query(self, params, bound_db=1.0, fallback=True):
        """Spectra for parameter rows: the surrogate where its estimated error
        is within bound_db, the DG runs it was trained on for the rest (when
        fallback is set). Returns (spectra, from_dg mask, estimated error)."""
        mean, est = self.predict(params)
        from_dg = est > bound_db
        if fallback and from_dg.any():
            P = np.asarray(params, dtype=np.float64).reshape(-1, 6)
            mean[from_dg], _ = dg_spectra(P[from_dg], steps=self.steps, grid=self.grid)
        return mean, from_dg, est

    def save(self, path):
        """Weights as their BF16 values (what the forward pass uses, so a
        loaded surrogate answers exactly as this one), biases and the
        normalisation in FP32."""
        params = np.stack([n.get_params() for n in self.nets])
        wmask = _weight_mask(WIDTHS)
        w16 = (_bf16_bits(params[:, wmask]) >> 16).astype(np.uint16)
        np.savez_compressed(path, weights_bf16=w16, biases=params[:, ~wmask], mu=self.mu, sigma=self.sigma,
                            scale=self.scale, widths=np.array(WIDTHS), grid=self.grid, steps=self.steps)

    @classmethod
    def load(cls, path, device=0):
        d = np.load(path)
        if list(d["widths"]) != WIDTHS:
            raise ValueError("network widths in %s differ from %s" % (path, WIDTHS))
        wmask = _weight_mask(WIDTHS)
        w16, b = d["weights_bf16"], d["biases"]
        params = np.zeros((w16.shape[0], wmask.size), dtype=np.float32)
        params[:, wmask] = (w16.astype(np.uint32) << 16).view(np.float32)
        params[:, ~wmask] = b
        return cls(list(params), d["mu"], float(d["sigma"]), float(d["scale"]), int(d["grid"]), int(d["steps"]),
                   device=device)

    def close(self):
        for n in self.nets:
            n.close()


def _weight_mask(widths):
    """True at the weight entries of the flat parameter vector (False at the
    biases)."""
    m = []
    for k, n in zip(widths[:-1], widths[1:]):
        m += [np.ones(n * k, dtype=bool), np.zeros(n, dtype=bool)]
    return np.concatenate(m)


def _bf16_bits(x):
    """uint32 bit patterns of float32 values rounded to BF16 (ties to even),
    as the GPU rounds its master weights."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)


def _init(widths, seed):
    """He-normal weights, zero biases (float32 flat vector)."""
    rng = np.random.default_rng(seed)
    flat = []
    for k, n in zip(widths[:-1], widths[1:]):
        flat += [rng.normal(0.0, math.sqrt(2.0 / k), size=n * k), np.zeros(n)]
    return np.concatenate(flat).astype(np.float32)

"""Learned spectral surrogate of the batched DG ensemble.

Maps the parameters of one 2-D LEE instance -- monopole position (x, y),
frequency f, mean-flow Mach number M and angle th, element order p -- to the
log power spectral density of the pressure at the ensemble's four observers
(128 bins each), with a fully connected network (6 -> 4 x 256 GELU -> 512,
BF16 weights, FP32 accumulation) that is trained and evaluated on the GPU by
the project's own kernels (gpu.Network, csrc/mlp.cu).

The reference has no counterpart: it answers every query with a DG run. DG
stays the measure of the network's error and its fallback here: the
training and test targets come from batched DG runs, and a query whose
estimated spectral error is above its bound's acceptance threshold is re-run
through DG. The estimate comes from an error network (6 -> 2 x 128 GELU -> 1,
the same kernels) trained on the logarithm of out-of-fold errors: networks
trained like the members, each without one fold of the training rows,
predict the fold they did not see. A calibration split's estimates and true
errors set each bound's threshold: the largest estimate under which at most
5 % of the accepted calibration queries exceed the bound.

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
ERR_WIDTHS = [6, 128, 128, 1]  # the error network
ERR_STEPS, ERR_LR, ERR_WEIGHT_DECAY = 4000, 2e-3, 0.01
RISK = 0.05  # largest share of accepted calibration queries above the bound
MIN_ACCEPT = 20  # calibration queries an acceptance threshold rests on


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


def accept_threshold(est, err, bound_db, risk=None, min_count=None):
    """Acceptance threshold on the estimated error for a bound: the largest
    calibration estimate t such that, of the calibration queries with an
    estimate <= t (at least min_count of them), at most the share `risk` has
    a true error above bound_db; +inf when the whole calibration split meets
    that, -inf when no prefix does (every query goes to DG)."""
    risk = RISK if risk is None else risk
    min_count = MIN_ACCEPT if min_count is None else min_count
    est = np.asarray(est, dtype=np.float64).reshape(-1)
    err = np.asarray(err, dtype=np.float64).reshape(-1)
    if est.size == 0:
        return -np.inf
    o = np.argsort(est, kind="stable")
    es = est[o]
    n = np.arange(1, es.size + 1)
    above = np.cumsum(err[o] > bound_db)
    # a threshold between two distinct estimates (ties stay together)
    ok = (above <= risk * n) & (n >= min_count) & np.append(es[1:] > es[:-1], True)
    if not ok.any():
        return -np.inf
    k = int(np.nonzero(ok)[0][-1])
    return np.inf if k == es.size - 1 else float(es[k])


class Surrogate:
    """Independently trained networks (four by default) whose mean answers a
    query, the target normalisation, the error network (the query's RMS
    error in dB, learned from out-of-fold errors of networks trained like
    the members) and a calibration split's estimates and true errors, which
    set each bound's acceptance threshold (accept_threshold)."""

    def __init__(self, params_list, mu, sigma, err_params, err_mu, err_sigma, calib_est=None, calib_err=None,
                 grid=GRID, steps=STEPS, device=0):
        self.mu = np.asarray(mu, dtype=np.float32)
        self.sigma = float(sigma)
        self.err_mu, self.err_sigma = float(err_mu), float(err_sigma)
        self.calib_est = np.zeros(0) if calib_est is None else np.asarray(calib_est, dtype=np.float64)
        self.calib_err = np.zeros(0) if calib_err is None else np.asarray(calib_err, dtype=np.float64)
        self.grid, self.steps = int(grid), int(steps)  # the DG runs the targets came from
        gpu = _pkg().gpu
        self.nets = []
        for p in params_list:
            net = gpu.Network(WIDTHS, device=device)
            net.set_params(p)
            self.nets.append(net)
        self.err_net = gpu.Network(ERR_WIDTHS, device=device)
        self.err_net.set_params(err_params)

    @classmethod
    def fit(cls, params, targets, n_models=4, steps=10000, batch=256, lr=4e-3, lr_final=2e-5, seed=0, grid=GRID,
            dg_steps=STEPS, weight_decay=0.1, err_steps=ERR_STEPS, device=0):
        """Members on all rows; then max(n_models, 2) networks with the same
        settings, each without one fold of the rows (row index modulo the
        fold count), give every row an out-of-fold RMS error, and the error
        network learns its logarithm."""
        gpu = _pkg().gpu
        x = features(params)
        y = np.asarray(targets, dtype=np.float64).reshape(len(x), -1)
        mu = y.mean(axis=0)
        sigma = float((y - mu).std())
        t = ((y - mu) / sigma).astype(np.float32)
        rng = np.random.default_rng(seed)

        def train(widths, rows, target, n_steps, lr0, wd):
            net = gpu.Network(widths, device=device)
            net.set_params(_init(widths, int(rng.integers(1 << 30))))
            net.set_data(x[rows], target[rows])
            loss = net.train(n_steps, batch, lr0, lr_final, seed=int(rng.integers(1 << 62)), weight_decay=wd)
            return net, loss

        everything = np.arange(len(x))
        plist, losses = [], []
        for _ in range(n_models):
            net, loss = train(WIDTHS, everything, t, steps, lr, weight_decay)
            plist.append(net.get_params())
            losses.append(loss)
            net.close()
        k_folds = max(n_models, 2)
        fold = everything % k_folds
        oof = np.zeros_like(y)
        for k in range(k_folds):
            net, _ = train(WIDTHS, np.nonzero(fold != k)[0], t, steps, lr, weight_decay)
            oof[fold == k] = net.forward(x[fold == k]).astype(np.float64) * sigma + mu
            net.close()
        le = np.log(np.maximum(rms_db(oof, y), 1e-6))
        err_mu, err_sigma = float(le.mean()), float(max(le.std(), 1e-6))
        te = ((le - err_mu) / err_sigma).astype(np.float32).reshape(-1, 1)
        enet, eloss = train(ERR_WIDTHS, everything, te, err_steps, ERR_LR, ERR_WEIGHT_DECAY)
        s = cls(plist, mu, sigma, enet.get_params(), err_mu, err_sigma, grid=grid, steps=dg_steps, device=device)
        enet.close()
        s.train_losses = losses
        s.err_train_loss = eloss
        s.oof_rms_db = np.exp(le)
        return s

    def predict(self, params):
        """Mean prediction [n][N_OBS][N_BINS] (dB) and the estimated RMS error
        per query (dB)."""
        x = features(params)
        ys = [net.forward(x).astype(np.float64) * self.sigma + self.mu for net in self.nets]
        mean = np.mean(ys, axis=0)
        est = np.exp(self.err_net.forward(x)[:, 0].astype(np.float64) * self.err_sigma + self.err_mu)
        return mean.reshape(-1, N_OBS, N_BINS), est

    def calibrate(self, params, targets):
        """Keep the estimates and true errors of these (held-out) queries:
        they set each bound's acceptance threshold. Returns the median true
        error."""
        mean, est = self.predict(params)
        self.calib_est = est
        self.calib_err = rms_db(mean, targets)
        return float(np.median(self.calib_err))

    def threshold(self, bound_db):
        """Largest estimated error accepted under bound_db (accept_threshold
        over the calibration split; -inf before calibration)."""
        if bound_db == np.inf:
            return np.inf
        return accept_threshold(self.calib_est, self.calib_err, bound_db)

    def query(self, params, bound_db=1.0, fallback=True):
        """Spectra for parameter rows: the surrogate where its estimated error
        is within the bound's acceptance threshold, the DG runs it was
        trained on for the rest (when fallback is set). Returns (spectra,
        from_dg mask, estimated error)."""
        mean, est = self.predict(params)
        from_dg = est > self.threshold(bound_db)
        if fallback and from_dg.any():
            P = np.asarray(params, dtype=np.float64).reshape(-1, 6)
            mean[from_dg], _ = dg_spectra(P[from_dg], steps=self.steps, grid=self.grid)
        return mean, from_dg, est

    def save(self, path):
        """Weights as their BF16 values (what the forward pass uses, so a
        loaded surrogate answers exactly as this one), biases, the
        normalisations and the calibration split in FP32/FP64."""
        params = np.stack([n.get_params() for n in self.nets])
        wmask = _weight_mask(WIDTHS)
        w16 = (_bf16_bits(params[:, wmask]) >> 16).astype(np.uint16)
        ep = self.err_net.get_params()
        emask = _weight_mask(ERR_WIDTHS)
        np.savez_compressed(path, weights_bf16=w16, biases=params[:, ~wmask], mu=self.mu, sigma=self.sigma,
                            err_weights_bf16=(_bf16_bits(ep[emask]) >> 16).astype(np.uint16), err_biases=ep[~emask],
                            err_mu=self.err_mu, err_sigma=self.err_sigma, calib_est=self.calib_est,
                            calib_err=self.calib_err, widths=np.array(WIDTHS), err_widths=np.array(ERR_WIDTHS),
                            grid=self.grid, steps=self.steps)

    @classmethod
    def load(cls, path, device=0):
        d = np.load(path)
        if list(d["widths"]) != WIDTHS:
            raise ValueError("network widths in %s differ from %s" % (path, WIDTHS))
        if "err_widths" not in d or list(d["err_widths"]) != ERR_WIDTHS:
            raise ValueError("%s holds no error network of widths %s" % (path, ERR_WIDTHS))

        def unpack(w16, b, widths):
            mask = _weight_mask(widths)
            w16 = np.atleast_2d(w16)
            p = np.zeros((w16.shape[0], mask.size), dtype=np.float32)
            p[:, mask] = (w16.astype(np.uint32) << 16).view(np.float32)
            p[:, ~mask] = np.atleast_2d(b)
            return p

        params = unpack(d["weights_bf16"], d["biases"], WIDTHS)
        ep = unpack(d["err_weights_bf16"], d["err_biases"], ERR_WIDTHS)[0]
        return cls(list(params), d["mu"], float(d["sigma"]), ep, float(d["err_mu"]), float(d["err_sigma"]),
                   d["calib_est"], d["calib_err"], int(d["grid"]), int(d["steps"]), device=device)

    def close(self):
        for n in self.nets:
            n.close()
        if getattr(self, "err_net", None) is not None:
            self.err_net.close()


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

"""Learned surrogate of the absorption factor with a traced audit.

``Surrogate``            an ensemble of MLPs (x7 -> 64 Fourier features -> 4 x 256 GELU
                         -> log A_h), trained and evaluated by the library's tensor-core
                         kernels (BF16 weights and activations, FP32 accumulation);
``inputs(...)``          the 7 network inputs of reflections (omega / 2pi and the incident and
                         diffracted unit vectors in the crystal frame);
``training_set(...)``    reflections drawn like the sample's and traced by the plain kernel;
``audited_absorption``   surrogate A_h with a seeded random audit fraction and every
                         high-spread reflection re-traced by the plain kernel, whose values
                         replace the surrogate's; the audit gives the error quantiles.

The ray tracer stays the reference: nothing here changes ``tracer``'s results.
"""
from __future__ import annotations

import ctypes as ct
import dataclasses

import numpy as np

from . import _lib, synth, tracer

N_FEATURES = 64
WIDTH = 256
DEPTH = 4


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def inputs(omega, s1, xray, omega_axis, F) -> np.ndarray:
    """[n][7] float32 network inputs of reflections, computed on the GPU."""
    L = _lib.load()
    s1 = _c(s1, np.float64).reshape(-1, 3)
    n = s1.shape[0]
    x7 = np.zeros((max(n, 1), 7), dtype=np.float32)
    _lib.check(L.anacor_surrogate_inputs(_c(omega, np.float64), s1, n, _c(xray, np.float64),
                                         _c(omega_axis, np.float64), _c(F, np.float64).reshape(-1), x7), L)
    return x7[:n]


def sample_inputs(s: synth.Sample) -> np.ndarray:
    return inputs(s.omega, s.s1, s.xray, s.omega_axis, s.F)


def tc_gemm(A: np.ndarray, B: np.ndarray, ksplit: int = 1) -> np.ndarray:
    """C[z] = bf16(A[z]) bf16(B[z])^T through the surrogate's tensor-core GEMM."""
    L = _lib.load()
    A = _c(A, np.float32)
    B = _c(B, np.float32)
    if A.ndim == 2:
        A, B = A[None], B[None]
    z, M, K = A.shape
    N = B.shape[1]
    C = np.zeros((z, M, N), dtype=np.float32)
    _lib.check(L.anacor_tc_gemm_check(A, B, M, N, K, z, int(ksplit), C), L)
    return C


class Surrogate:
    """Ensemble of ``members`` networks living on the current CUDA device."""

    def __init__(self, members: int = 4, seed: int = 0, fourier_scale: float = 0.5):
        self._L = _lib.load()
        h = self._L.anacor_surrogate_create(int(members), int(seed) & 0xFFFFFFFF, float(fourier_scale))
        if not h:
            raise _lib.AnacorError(*_lib.last_error(self._L))
        self._h = ct.c_void_p(h)
        self.members = int(members)
        self.param_count = int(self._L.anacor_surrogate_param_count())
        self.steps_done = 0

    # ---------------------------------------------------------- parameters
    def get_params(self) -> np.ndarray:
        p = np.zeros((self.members, self.param_count), dtype=np.float32)
        _lib.check(self._L.anacor_surrogate_params(self._h, p, 0), self._L)
        return p

    def set_params(self, p: np.ndarray):
        p = _c(p, np.float32).reshape(self.members, self.param_count)
        _lib.check(self._L.anacor_surrogate_params(self._h, p, 1), self._L)

    def get_fourier(self) -> np.ndarray:
        b = np.zeros((32, 7), dtype=np.float32)
        _lib.check(self._L.anacor_surrogate_fourier(self._h, b, 0), self._L)
        return b

    def set_fourier(self, b: np.ndarray):
        _lib.check(self._L.anacor_surrogate_fourier(self._h, _c(b, np.float32).reshape(32, 7), 1), self._L)

    @property
    def scale(self) -> tuple[float, float]:
        m, s = ct.c_double(), ct.c_double()
        _lib.check(self._L.anacor_surrogate_scale(self._h, ct.byref(m), ct.byref(s), 0), self._L)
        return m.value, s.value

    @scale.setter
    def scale(self, ms):
        m, s = ct.c_double(ms[0]), ct.c_double(ms[1])
        _lib.check(self._L.anacor_surrogate_scale(self._h, ct.byref(m), ct.byref(s), 1), self._L)

    # ------------------------------------------------------------ training
    def set_data(self, x7: np.ndarray, log_ah: np.ndarray):
        x7 = _c(x7, np.float32).reshape(-1, 7)
        _lib.check(self._L.anacor_surrogate_set_data(self._h, x7, _c(log_ah, np.float64), x7.shape[0]), self._L)

    def train(self, steps: int, batch: int = 4096, lr_max: float = 3e-3, lr_min: float = 3e-5,
              total_steps: int | None = None) -> np.ndarray:
        """Adam steps on the training set; returns the mean member loss of each step."""
        loss = np.zeros(max(steps, 1), dtype=np.float32)
        total = int(total_steps if total_steps is not None else self.steps_done + steps)
        _lib.check(self._L.anacor_surrogate_train(self._h, int(steps), int(batch), float(lr_max), float(lr_min),
                                                  total, loss.ctypes.data), self._L)
        self.steps_done += steps
        return loss[:steps]

    def gradients(self, x7: np.ndarray, target: np.ndarray):
        """Loss gradients of every member on one batch (targets in output units);
        returns (grads [members][param_count], y [members][rows])."""
        x7 = _c(x7, np.float32).reshape(-1, 7)
        rows = x7.shape[0]
        g = np.zeros((self.members, self.param_count), dtype=np.float32)
        y = np.zeros((self.members, rows), dtype=np.float32)
        _lib.check(self._L.anacor_surrogate_gradients(self._h, x7, _c(target, np.float32), rows, g.ctypes.data,
                                                      y.ctypes.data), self._L)
        return g, y

    # ----------------------------------------------------------- inference
    def predict(self, x7: np.ndarray, members: bool = False):
        """(mean A_h, relative spread[, per-member log A_h]) of n rows of x7."""
        x7 = _c(x7, np.float32).reshape(-1, 7)
        n = x7.shape[0]
        mean = np.zeros(max(n, 1), dtype=np.float32)
        spread = np.zeros(max(n, 1), dtype=np.float32)
        mem = np.zeros((self.members, max(n, 1)), dtype=np.float32) if members else None
        _lib.check(self._L.anacor_surrogate_predict(self._h, x7, n, mean, spread,
                                                    mem.ctypes.data if mem is not None else None), self._L)
        if members:
            return mean[:n], spread[:n], mem[:, :n]
        return mean[:n], spread[:n]

    def set_inference(self, fused: bool = True):
        """Fused (one persistent kernel, activations on chip; the default) or
        layer-by-layer inference; the same numbers either way."""
        _lib.check(self._L.anacor_surrogate_set_inference(self._h, 1 if fused else 0), self._L)

    def predict_device(self, d_x7: int, n: int, d_mean: int, d_spread: int, stream: int | None = None,
                       d_members: int | None = None):
        """Enqueue inference on device buffers (raw pointers) on `stream`."""
        _lib.check(self._L.anacor_surrogate_predict_device(self._h, ct.c_void_p(d_x7), int(n), ct.c_void_p(d_mean),
                                                           ct.c_void_p(d_spread), ct.c_void_p(d_members or 0),
                                                           ct.c_void_p(stream or 0)), self._L)

    # --------------------------------------------------------- checkpoints
    def save(self, path: str):
        _lib.check(self._L.anacor_surrogate_save(self._h, str(path).encode()), self._L)

    def load(self, path: str):
        _lib.check(self._L.anacor_surrogate_load(self._h, str(path).encode()), self._L)

    def close(self):
        if getattr(self, "_h", None):
            self._L.anacor_surrogate_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def audit_flags(d_spread: int, n: int, seed: int, fraction: float, threshold: float, d_flags: int,
                stream: int | None = None):
    L = _lib.load()
    _lib.check(L.anacor_surrogate_audit_flags(ct.c_void_p(d_spread), int(n), int(seed) & 0xFFFFFFFF,
                                              float(fraction), float(threshold), ct.c_void_p(d_flags),
                                              ct.c_void_p(stream or 0)), L)


def audit_flags_host(spread: np.ndarray, seed: int, fraction: float, threshold: float) -> np.ndarray:
    """The audit flags of host spreads (same rule and hash as the device kernel)."""
    import torch   # device buffers for the one kernel call

    sp = torch.as_tensor(_c(spread, np.float32), device="cuda")
    fl = torch.empty(sp.shape[0], dtype=torch.uint8, device="cuda")
    audit_flags(sp.data_ptr(), sp.shape[0], seed, fraction, threshold, fl.data_ptr(),
                torch.cuda.current_stream().cuda_stream)
    return fl.cpu().numpy()


def training_set(s: synth.Sample, n: int = 100_000, seed: int = 7, plan: tracer.Plan | None = None):
    """n reflections drawn as the sample's (omega uniform, 2theta in [5, 120] deg,
    uniform azimuth) and traced by the plain kernel: (omega, s1, A_h)."""
    rng = np.random.default_rng(seed)
    omega, s1 = synth.reflections(n, rng, xray=s.xray)
    own = plan is None
    p = plan or tracer.Plan(s.label, s.coords, s.voxel, s.mu)
    try:
        p.set_reflections(s1, omega, s.xray, s.omega_axis, s.F)
        p.run()
        ah = p.result()
    finally:
        if own:
            p.close()
    return omega, s1, ah


@dataclasses.dataclass
class AuditResult:
    ah: np.ndarray            # final A_h: surrogate, replaced by traced values where traced
    surrogate: np.ndarray     # the ensemble mean for every reflection
    spread: np.ndarray
    flags: np.ndarray         # bit 0 random audit, bit 1 spread above threshold
    traced_idx: np.ndarray
    traced: np.ndarray

    @property
    def audit_rel_err(self) -> np.ndarray:
        """|surrogate - traced| / traced on the random audit sample."""
        sel = (self.flags[self.traced_idx] & 1) != 0
        t = self.traced[sel]
        return np.abs(self.surrogate[self.traced_idx[sel]].astype(np.float64) - t) / np.abs(t)

    def quantiles(self, q=(0.5, 0.9, 0.99, 1.0)) -> dict:
        e = self.audit_rel_err
        if e.size == 0:
            return {}
        return {f"q{int(round(x * 100))}": float(np.quantile(e, x)) for x in q}

    @property
    def fallback_fraction(self) -> float:
        return float(np.mean((self.flags & 2) != 0)) if self.flags.size else 0.0


def audited_absorption(model: Surrogate, plan: tracer.Plan, omega, s1, xray, omega_axis, F,
                       audit_fraction: float = 0.02, spread_threshold: float = 1e-3, seed: int = 0) -> AuditResult:
    """Surrogate A_h of the reflections, with the audit rows and the high-spread
    rows re-traced by ``plan`` (the plain kernel) and their traced values kept."""
    omega = _c(omega, np.float64)
    s1 = _c(s1, np.float64).reshape(-1, 3)
    x7 = inputs(omega, s1, xray, omega_axis, F)
    mean, spread = model.predict(x7)
    flags = audit_flags_host(spread, seed, audit_fraction, spread_threshold)
    idx = np.nonzero(flags)[0]
    traced = np.zeros(0)
    ah = mean.astype(np.float64)
    if idx.size:
        plan.set_reflections(s1[idx], omega[idx], xray, omega_axis, F)
        plan.run()
        traced = plan.result()
        ah[idx] = traced
    return AuditResult(ah=ah, surrogate=mean, spread=spread, flags=flags, traced_idx=idx, traced=traced)


def train_for_sample(s: synth.Sample, n_train: int = 100_000, steps: int = 20_000, batch: int = 4096,
                     members: int = 4, seed: int = 0, fourier_scale: float = 0.5, lr_max: float = 3e-3,
                     lr_min: float = 3e-5, plan: tracer.Plan | None = None):
    """Trace a training set on the sample and train an ensemble on it; returns
    (model, loss history)."""
    omega, s1, ah = training_set(s, n_train, seed=seed + 7, plan=plan)
    x7 = inputs(omega, s1, s.xray, s.omega_axis, s.F)
    model = Surrogate(members=members, seed=seed, fourier_scale=fourier_scale)
    model.set_data(x7, np.log(ah))
    loss = model.train(steps, batch=batch, lr_max=lr_max, lr_min=lr_min, total_steps=steps)
    return model, loss


def select_fourier_scale(x7: np.ndarray, log_ah: np.ndarray, candidates=(0.25, 0.35, 0.5),
                         steps: int = 3000, batch: int = 4096, members: int = 4, seed: int = 0,
                         lr_max: float = 3e-3, holdout: float = 0.1, spread_threshold: float = 1e-3):
    """Fourier feature scale for a training set, chosen on held-out rows.

    Each candidate ensemble trains for a short cosine schedule on all but the
    last ``holdout`` fraction of the rows; the held-out rows are predicted and
    the candidate with the fewest rows above ``spread_threshold`` (the rows the
    audit would re-trace) wins, ties broken by the median relative error.
    Returns (scale, {scale: (fallback fraction, median error)}).  A smaller
    scale gives smoother features: it wins on strongly absorbing samples,
    whose A_h varies more steeply with direction, where a larger scale
    leaves the members disagreeing on more rows."""
    x7 = _c(x7, np.float32).reshape(-1, 7)
    log_ah = _c(log_ah, np.float64)
    n = x7.shape[0]
    n_fit = max(1, int(round(n * (1.0 - holdout))))
    if n_fit >= n:
        raise ValueError("select_fourier_scale needs held-out rows")
    target = np.exp(log_ah[n_fit:])
    scores = {}
    for fs in candidates:
        m = Surrogate(members=members, seed=seed, fourier_scale=float(fs))
        try:
            m.set_data(x7[:n_fit], log_ah[:n_fit])
            m.train(steps, batch=batch, lr_max=lr_max, lr_min=lr_max * 1e-2, total_steps=steps)
            mean, spread = m.predict(x7[n_fit:])
        finally:
            m.close()
        fb = float(np.mean(~(spread <= spread_threshold)))
        scores[float(fs)] = (fb, float(np.median(relative_error(mean, target))))
    best = min(scores, key=lambda k: scores[k])
    return best, scores


def relative_error(a, b) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.abs(b)


__all__ = ["Surrogate", "inputs", "sample_inputs", "tc_gemm", "training_set", "audited_absorption",
           "AuditResult", "train_for_sample", "select_fourier_scale", "audit_flags", "audit_flags_host", "relative_error",
           "N_FEATURES", "WIDTH", "DEPTH"]

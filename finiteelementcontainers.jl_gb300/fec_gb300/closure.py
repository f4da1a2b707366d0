"""The learned J2 closure: training data from the exact return map, training
with the library's hand-written kernels, and the physics that uses it.

Features (physical units; the network sees them normalised by the data's mean
and standard deviation):
  input  (14): elastic trial strain e_tr = eps - eps_p_old (xx yy zz yz xz xy, tensor
               components), eps_p_old (6), eqps_old (1), yield flag (1)
  output (13): plastic correction of the deviatoric stress, s - 2 mu dev(e_tr) (6), plastic
               strain increment (6), eqps increment (1); the elastic trial deviator and the
               pressure kappa tr(e_tr) are exact for J2 (plastic flow is deviatoric) and are
               added outside the network
The closure serves plastic points only: elastic points are exact and cheap, and
a plastic point whose predicted stress misses the updated yield surface by more
than `tol * sigma_y` falls back to the exact radial return."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .physics import AbstractPhysics

IN, OUT = 14, 13


def _torch():
    import torch
    return torch


def exact_points(props, strain, state_old, want_tangent: bool = False):
    """Exact J2 return map of a batch (device float64 tensors): (stress, state_new, tangent or None)."""
    torch = _torch()
    lib = _lib.load()
    n = strain.shape[0]
    stress = torch.empty(n, 6, dtype=torch.float64, device=strain.device)
    st_new = torch.empty(n, 7, dtype=torch.float64, device=strain.device)
    tan = torch.empty(n, 6, 6, dtype=torch.float64, device=strain.device) if want_tangent else None
    pr = np.ascontiguousarray(props, dtype=np.float64)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.fec_j2_points(_lib.ptr(pr), n, _lib.ptr(strain.contiguous()), _lib.ptr(state_old.contiguous()),
                           _lib.ptr(stress), _lib.ptr(st_new), _lib.ptr(tan), stream)
    if st != 0:
        raise _lib.FECError(st, "fec_j2_points failed")
    return stress, st_new, tan


def deviatoric(s6):
    """Deviatoric part of stresses in Voigt order xx yy zz yz xz xy."""
    torch = _torch()
    p = s6[:, :3].mean(1, keepdim=True)
    return s6 - torch.cat([p, p, p, 0 * p, 0 * p, 0 * p], 1)


def elastic_deviator(props, etr):
    """Elastic trial deviator 2 mu dev(e_tr), Voigt order, tensor shear components."""
    E, nu = props[0], props[1]
    return 2 * E / (2 * (1 + nu)) * deviatoric(etr)


def deviatoric_stress(props, X, out):
    """Deviatoric stress of network-layout rows `out` (correction + exact trial deviator)."""
    return out[:, :6] + elastic_deviator(props, X[:, :6])


def pressure(props, etr):
    """Exact J2 pressure kappa tr(e_tr)."""
    E, nu = props[0], props[1]
    return E / (3 * (1 - 2 * nu)) * etr[:, :3].sum(1, keepdim=True)


def yield_flag(props, etr, eqps):
    """1 where the elastic trial state violates the yield condition."""
    E, nu, sy, H = props
    mu = E / (2 * (1 + nu))
    tr = etr[:, :3].sum(1, keepdim=True)
    dev = 2 * mu * (etr - _torch().cat([tr / 3.0, tr / 3.0, tr / 3.0, 0 * tr, 0 * tr, 0 * tr], 1))
    w = _torch().tensor([1, 1, 1, 2, 2, 2], dtype=etr.dtype, device=etr.device)
    f = (dev * dev * w).sum(1).sqrt() - np.sqrt(2.0 / 3.0) * (sy + H * eqps)
    return (f > 0).to(etr.dtype)


def sample_rows(props, eps, state_old, stress, state_new):
    """Network input and target rows of return-map results: strain eps (tensor
    components), state before and after, stress (Voigt)."""
    torch = _torch()
    etr = eps - state_old[:, :6]
    flag = yield_flag(props, etr, state_old[:, 6])
    X = torch.cat([etr, state_old, flag[:, None]], 1)
    Y = torch.cat([deviatoric(stress) - elastic_deviator(props, etr), state_new - state_old], 1)
    return X, Y


def generate_samples(props, n_paths: int, steps: int = 20, max_strain: float = 0.02, seed: int = 4,
                     device: str = "cuda"):
    """Samples along random strain paths through the exact return map.  Half the
    paths are proportional (one direction), half non-proportional (the direction
    turns to a second random direction halfway).  Returns (X, Y, plastic mask)
    float64 tensors with one row per (path, step)."""
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    d1 = torch.randn(n_paths, 6, generator=g, dtype=torch.float64)
    d2 = torch.randn(n_paths, 6, generator=g, dtype=torch.float64)
    d1 /= d1.norm(dim=1, keepdim=True)
    d2 /= d2.norm(dim=1, keepdim=True)
    amp = max_strain * torch.rand(n_paths, 1, generator=g, dtype=torch.float64)
    nonprop = torch.arange(n_paths) % 2 == 1
    d1, d2, amp = d1.to(device), d2.to(device), amp.to(device)
    state = torch.zeros(n_paths, 7, dtype=torch.float64, device=device)
    eps = torch.zeros(n_paths, 6, dtype=torch.float64, device=device)
    Xs, Ys, Ps = [], [], []
    for s in range(1, steps + 1):
        turn = nonprop.to(device) & (s > steps // 2)
        dirn = torch.where(turn[:, None], d2, d1)
        eps = eps + amp * dirn / steps
        stress, new, _ = exact_points(props, eps, state)
        x, y = sample_rows(props, eps, state, stress, new)
        Xs.append(x)
        Ys.append(y)
        Ps.append(x[:, 13] > 0)
        state = new
    return torch.cat(Xs), torch.cat(Ys), torch.cat(Ps)


@dataclass
class TrainedClosure:
    params: np.ndarray          # FP32, the library's layout
    normalisation: np.ndarray   # 14 + 14 + 13 + 13 floats: in mean, in std, out mean, out std
    history: list
    tol: float = 1e-4

    def normalise_in(self, X):
        m, s = self.normalisation[:IN], self.normalisation[IN:2 * IN]
        return (X - _torch().as_tensor(m, device=X.device)) / _torch().as_tensor(s, device=X.device)

    def predict(self, X):
        """Network output in physical units (FP32 parameters; X float64/32 tensor on the device)."""
        torch = _torch()
        lib = _lib.load()
        Xn = self.normalise_in(X.to(torch.float64)).float().contiguous()
        Y = torch.empty(X.shape[0], OUT, dtype=torch.float32, device=X.device)
        p = torch.from_numpy(self.params).to(X.device)
        st = lib.fec_mlp_forward(_lib.ptr(p), _lib.ptr(Xn), X.shape[0], _lib.ptr(Y),
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
        if st != 0:
            raise _lib.FECError(st, "fec_mlp_forward failed")
        om = torch.as_tensor(self.normalisation[2 * IN:2 * IN + OUT], device=X.device)
        os_ = torch.as_tensor(self.normalisation[2 * IN + OUT:], device=X.device)
        return Y.double() * os_ + om


def consistency_residual(props, X, pred):
    """|f| / sigma_y of network-layout rows `pred` (deviatoric-stress correction, state
    increment): the distance of the predicted stress from the updated yield surface."""
    torch = _torch()
    E, nu, sy, H = props
    dev = deviatoric_stress(props, X, pred)
    w = torch.tensor([1, 1, 1, 2, 2, 2], dtype=dev.dtype, device=dev.device)
    eqps = X[:, 12] + pred[:, 12]
    f = (dev * dev * w).sum(1).sqrt() - np.sqrt(2.0 / 3.0) * (sy + H * eqps)
    return f.abs() / sy


def validation_errors(trained: TrainedClosure, props, X, Y, tols=(1e-4, 1e-3, 1e-2)) -> dict:
    """Held-out errors of the network with its FP32 parameters and with the BF16
    rounding the assembly uses: relative stress error (full and deviatoric),
    state-increment error, and the share of points that pass the consistency
    check at each tolerance."""
    torch = _torch()
    pres = pressure(props, X[:, :6])
    sdev = lambda o: deviatoric_stress(props, X, o)  # noqa: E731
    full = lambda o: sdev(o) + torch.cat([pres, pres, pres, 0 * pres, 0 * pres, 0 * pres], 1)  # noqa: E731
    out = {}
    bf16 = torch.from_numpy(trained.params).bfloat16().float().numpy()
    for name, params in (("fp32_params", trained.params), ("bf16_params", bf16)):
        pv = TrainedClosure(params, trained.normalisation, []).predict(X)
        cres = consistency_residual(props, X, pv)
        out[name] = {
            "stress": float((full(pv) - full(Y)).norm() / full(Y).norm()),
            "deviatoric_stress": float((sdev(pv) - sdev(Y)).norm() / sdev(Y).norm()),
            "state_increment": float((pv[:, 6:] - Y[:, 6:]).norm() / Y[:, 6:].norm()),
            "consistency_pass": {f"{t:g}": float((cres <= t).double().mean()) for t in tols}}
    out["points"] = int(X.shape[0])
    return out


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation in the library's parameter layout."""
    rng = np.random.default_rng(seed)
    dims = [IN, 64, 64, 64, 64, OUT]
    out = []
    for i in range(5):
        W = rng.standard_normal((dims[i + 1], dims[i])) * np.sqrt(2.0 / dims[i])
        out += [W.ravel(), np.zeros(dims[i + 1])]
    p = np.concatenate(out).astype(np.float32)
    assert p.size == _lib.load().fec_mlp_param_count()
    return p


def train(X, Y, epochs: int = 10, batch: int = 16384, lr: float = 2e-3, seed: int = 0, tol: float = 1e-4,
          log=None) -> TrainedClosure:
    """Adam on normalised features with the library's forward/backward/Adam kernels."""
    torch = _torch()
    lib = _lib.load()
    dev = X.device
    in_m, in_s = X.mean(0), X.std(0)
    out_m, out_s = Y.mean(0), Y.std(0)
    in_s = torch.where(in_s > 1e-12, in_s, torch.ones_like(in_s))
    out_s = torch.where(out_s > 1e-12, out_s, torch.ones_like(out_s))
    norm = torch.cat([in_m, in_s, out_m, out_s]).float().cpu().numpy()
    Xn = ((X - in_m) / in_s).float().contiguous()
    Yn = ((Y - out_m) / out_s).float().contiguous()
    P = torch.from_numpy(init_params(seed)).to(dev)
    m = torch.zeros_like(P)
    v = torch.zeros_like(P)
    nb = (batch + 63) // 64
    scratch = torch.empty(nb * (P.numel() + 1), dtype=torch.float32, device=dev)
    loss = torch.zeros(1, dtype=torch.float32, device=dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n = Xn.shape[0]
    step, history = 0, []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g).to(dev)
        rate = lr * (0.5 * (1 + np.cos(np.pi * ep / epochs)))  # cosine decay per epoch
        tot, cnt = 0.0, 0
        for s0 in range(0, n - batch + 1, batch):
            idx = perm[s0:s0 + batch]
            xb, yb = Xn.index_select(0, idx), Yn.index_select(0, idx)
            step += 1
            st = lib.fec_mlp_adam_step(_lib.ptr(P), _lib.ptr(m), _lib.ptr(v), _lib.ptr(xb), _lib.ptr(yb), batch,
                                       step, float(rate), _lib.ptr(scratch), scratch.numel(), _lib.ptr(loss), stream)
            if st != 0:
                raise _lib.FECError(st, "fec_mlp_adam_step failed")
            if s0 % (batch * 64) == 0:
                tot += float(loss)
                cnt += 1
        history.append(tot / max(cnt, 1))
        if log:
            log(f"epoch {ep}: loss {history[-1]:.3e}")
    return TrainedClosure(P.cpu().numpy(), norm, history, tol)


class J2Closure(AbstractPhysics):
    """J2 plasticity whose plastic points use a trained closure (FP32-element
    assembly of hex8 blocks); props as J2Plasticity."""
    NF, NP, NS, ID = 3, 4, 7, _lib.FEC_PHYS_J2_MLP

    def __init__(self, E: float, nu: float, yield_stress: float, hardening: float, closure: TrainedClosure):
        self.E, self.nu, self.sy, self.H = float(E), float(nu), float(yield_stress), float(hardening)
        self.closure = closure

    def create_properties(self):
        return np.array([self.E, self.nu, self.sy, self.H], dtype=np.float64)

    def install(self, asm) -> None:
        params = np.ascontiguousarray(self.closure.params, dtype=np.float32)
        norm = np.ascontiguousarray(self.closure.normalisation, dtype=np.float32)
        asm._call("fec_closure_set", _lib.ptr(params), _lib.ptr(norm), float(self.closure.tol))

    @staticmethod
    def stats(asm, reset: bool = False) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        asm._call("fec_closure_stats", C.byref(a), C.byref(b), int(reset))
        return a.value, b.value

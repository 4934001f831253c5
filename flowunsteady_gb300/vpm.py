"""FLOWVPM-shaped host API over libvpmgpu.so.

The names follow the FLOWVPM symbols that FLOWUnsteady passes around
(src/FLOWUnsteady_simulation.jl:107-253 of byuflowlab/FLOWUnsteady):

    pfield = ParticleField(max_particles; formulation=rVPM, viscous=Inviscid(),
                           kernel=gaussianerf, UJ=UJ_gpu, SFS=noSFS,
                           integration=rungekutta3, transposed=True,
                           relaxation=norelaxation, Uinf=...)
    add_particle(pfield, X, Gamma, sigma; vol=0, circulation=1, C=None, static=False)
    add_probe(pfield, X)                  (Γ = 0, σ = 1e-6, vol = 0; :572)
    add_shed_particles(pfield, X, gamma, dt, V, infD, sigma, vol, l, p_per_step)
                                          (FLOWUnsteady's shedding add_particle, :455-489)
    remove_particle(pfield, i)            (tail removal,     :360-365, :550-552)
    get_np(pfield)
    pfield.UJ(pfield)                     (probe / force evaluation, :544)
    nextstep(pfield, dt; relax=False)     (:358)
    monitor_enstrophy(pfield), monitor_Cd(pfield)   (src/FLOWUnsteady_monitors.jl:614,697)

Everything computes on the GPU through the C ABI; particle data lives in
device memory owned by the library.  Appends are buffered on the host and
uploaded before the next device call.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import _lib as L

# ------------------------------------------------------------------ kernels --


@dataclass(frozen=True)
class Kernel:
    """Regularising kernel (FLOWVPM's vpm.Kernel)."""
    name: str
    id: int

    def zeta0(self) -> float:
        return 15.0 / (8.0 * np.pi) if self.id == L.KERNEL_WINCKELMANS else (2 * np.pi) ** -1.5


winckelmans = Kernel("winckelmans", L.KERNEL_WINCKELMANS)
gaussianerf = Kernel("gaussianerf", L.KERNEL_GAUSSIANERF)

# -------------------------------------------------------------- formulation --


@dataclass(frozen=True)
class Formulation:
    """rVPM constants f, g (docs/src/theory/rvpm.md:196-237)."""
    f: float
    g: float


rVPM = Formulation(0.0, 0.2)
cVPM = Formulation(0.0, 0.0)

# ------------------------------------------------------------------ viscous --


@dataclass
class Inviscid:
    nu: float = 0.0


@dataclass
class CoreSpreading:
    """Viscous core spreading d(σ²)/dt = 2ν (vpm.CoreSpreading(nu, sgm0, zeta)).

    The RBF re-initialisation when σ outgrows beta·sgm0 is not provided."""
    nu: float
    sgm0: Optional[float] = None
    beta: float = 1.5


# ---------------------------------------------------------------------- SFS --


@dataclass
class NoSFS:
    pass


noSFS = NoSFS()
SFS_none = noSFS


def Estr_direct():
    """Marker of the direct E_str pair pass (vpm.Estr_direct)."""
    return "Estr_direct"


clipping_backscatter = "clipping_backscatter"
pseudo3level = "pseudo3level"
pseudo3level_positive = "pseudo3level_positive"


@dataclass
class DynamicSFS:
    """vpm.DynamicSFS(Estr_direct, procedure; alpha, rlxf, minC, maxC, clippings)."""
    model: object = Estr_direct
    procedure: str = pseudo3level_positive
    alpha: float = 0.999
    rlxf: float = 1.0
    minC: float = 0.0
    maxC: float = 1.0
    clippings: Sequence[str] = (clipping_backscatter,)


@dataclass
class ConstantSFS:
    """E_str with a prescribed coefficient C_d."""
    Cd: float
    clippings: Sequence[str] = (clipping_backscatter,)


# -------------------------------------------------------------- integration --
euler = "euler"
rungekutta3 = "rungekutta3"


@dataclass
class Relaxation:
    """Pedrizzetti relaxation (vpm.pedrizzetti): factor rlxf every nsteps_relax steps."""
    rlxf: float = 0.3
    nsteps_relax: int = 1


norelaxation = None
pedrizzetti = Relaxation()

# ----------------------------------------------------------------------- UJ --


def _uj(precision: int) -> Callable:
    def UJ(pfield: "ParticleField"):
        pfield._flush()
        L.check(L.lib().vpm_eval_UJ(pfield._ctx, pfield.kernel.id, precision), pfield._ctx)
        pfield._uj_valid = True
    UJ.precision = precision
    return UJ


UJ_direct = _uj(L.PREC_FP64)         # plain FP64 direct sum (the parity form)
UJ_gpu = _uj(L.PREC_FP32C)           # FP32 tile-relative compensated direct sum
UJ_gpu_fp32 = _uj(L.PREC_FP32)       # naive FP32 (precision studies only)

# -------------------------------------------------------------- the field --


class ParticleField:
    """Device-resident particle field (FLOWVPM's vpm.ParticleField)."""

    def __init__(self, maxparticles: int, *, formulation: Formulation = rVPM,
                 viscous=None, kernel: Kernel = gaussianerf, UJ: Callable = UJ_gpu,
                 SFS=noSFS, integration: str = rungekutta3, transposed: bool = True,
                 relaxation: Optional[Relaxation] = norelaxation,
                 Uinf: Sequence[float] = (0.0, 0.0, 0.0), device: int = 0):
        self.maxparticles = int(maxparticles)
        self.formulation = formulation
        self.viscous = viscous if viscous is not None else Inviscid()
        self.kernel = kernel
        self.UJ = UJ
        self.SFS = SFS
        self.integration = integration
        self.transposed = transposed
        self.relaxation = relaxation
        self.Uinf = tuple(float(u) for u in Uinf)
        ptr = ctypes.c_void_p()
        L.check(L.lib().vpm_ctx_create(int(device), self.maxparticles, ctypes.byref(ptr)))
        self._ctx = ptr
        self._pend: List[tuple] = []
        self._uj_valid = False

    # -- lifetime
    def close(self):
        if getattr(self, "_ctx", None):
            L.lib().vpm_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particle_order(self, mode: int):
        """L.ORDER_AUTO (default: pair passes over fields of 65,536 particles or
        more run along a Morton curve of the positions) or L.ORDER_CALLER (the
        field's own order, as FLOWVPM sums); vpm_set_particle_order."""
        L.check(L.lib().vpm_set_particle_order(self._ctx, int(mode)), self._ctx)

    # -- scheme
    def scheme(self, precision: Optional[int] = None) -> L.Scheme:
        s = L.default_scheme()
        s.kernel = self.kernel.id
        s.precision = getattr(self.UJ, "precision", L.PREC_FP32C) if precision is None else precision
        s.integration = L.INTEGRATION_RK3 if self.integration == rungekutta3 else L.INTEGRATION_EULER
        s.transposed = 1 if self.transposed else 0
        s.f, s.g = self.formulation.f, self.formulation.g
        for k in range(3):
            s.uinf[k] = self.Uinf[k]
        s.nu = float(getattr(self.viscous, "nu", 0.0) or 0.0)
        if isinstance(self.SFS, DynamicSFS):
            s.sfs = L.SFS_DYNAMIC
            s.sfs_alpha, s.sfs_rlxf = self.SFS.alpha, self.SFS.rlxf
            s.sfs_minC, s.sfs_maxC = self.SFS.minC, self.SFS.maxC
            flags = L.SFS_CLIP_BACKSCATTER if clipping_backscatter in self.SFS.clippings else 0
            if self.SFS.procedure == pseudo3level_positive:
                flags |= L.SFS_FORCE_POSITIVE
            s.sfs_flags = flags
        elif isinstance(self.SFS, ConstantSFS):
            s.sfs = L.SFS_CONSTANT
            s.sfs_Cd = self.SFS.Cd
            s.sfs_flags = L.SFS_CLIP_BACKSCATTER if clipping_backscatter in self.SFS.clippings else 0
        else:
            s.sfs = L.SFS_NONE
        if self.relaxation is not None:
            s.relaxation = L.RELAX_PEDRIZZETTI
            s.relax_factor = self.relaxation.rlxf
            s.relax_nsteps = self.relaxation.nsteps_relax
        return s

    # -- particles
    def _flush(self):
        if not self._pend:
            return
        # Consecutive appends with the same static flag go up in one call.
        groups = []
        for X, G, S, static, attrs in self._pend:
            if groups and groups[-1][3] == static:
                g = groups[-1]
                g[0].append(X); g[1].append(G); g[2].append(S); g[4].append(attrs)
            else:
                groups.append(([X], [G], [S], static, [attrs]))
        self._pend = []
        for Xs, Gs, Ss, static, attrs in groups:
            X = np.ascontiguousarray(np.concatenate(Xs), dtype=np.float64)
            G = np.ascontiguousarray(np.concatenate(Gs), dtype=np.float64)
            S = np.ascontiguousarray(np.concatenate(Ss), dtype=np.float64)
            n0 = self._np_device()
            L.check(L.lib().vpm_append(self._ctx, X.shape[0], L.dptr(X), 3, L.dptr(G), 3,
                                       L.dptr(S), 1, 1 if static else 0), self._ctx)
            # vol / circulation / C other than the defaults (0, 1, 0).
            if any(a is not None for a in attrs):
                vol = np.concatenate([a[0] if a else np.zeros(x.shape[0])
                                      for a, x in zip(attrs, Xs)])
                circ = np.concatenate([a[1] if a else np.ones(x.shape[0])
                                       for a, x in zip(attrs, Xs)])
                C = np.concatenate([a[2] if a else np.zeros((x.shape[0], 3))
                                    for a, x in zip(attrs, Xs)])
                vol, circ, C = (np.ascontiguousarray(v, dtype=np.float64) for v in (vol, circ, C))
                L.check(L.lib().vpm_set_attributes(self._ctx, n0, X.shape[0], L.dptr(vol), 1,
                                                   L.dptr(circ), 1, L.dptr(C), 3), self._ctx)
        self._uj_valid = False

    def _np_device(self) -> int:
        n = ctypes.c_int64()
        L.check(L.lib().vpm_get_np(self._ctx, ctypes.byref(n), None), self._ctx)
        return int(n.value)

    def set_particles(self, X, Gamma, sigma):
        self._pend = []
        X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        G = np.ascontiguousarray(Gamma, dtype=np.float64).reshape(-1, 3)
        S = np.ascontiguousarray(sigma, dtype=np.float64).reshape(-1)
        L.check(L.lib().vpm_set_particles(self._ctx, X.shape[0], L.dptr(X), 3, L.dptr(G), 3,
                                          L.dptr(S), 1), self._ctx)
        self._uj_valid = False

    def get_np(self) -> int:
        self._flush()
        n = ctypes.c_int64()
        ns = ctypes.c_int64()
        L.check(L.lib().vpm_get_np(self._ctx, ctypes.byref(n), ctypes.byref(ns)), self._ctx)
        return int(n.value)

    def get_nstatic(self) -> int:
        self._flush()
        n = ctypes.c_int64()
        ns = ctypes.c_int64()
        L.check(L.lib().vpm_get_np(self._ctx, ctypes.byref(n), ctypes.byref(ns)), self._ctx)
        return int(ns.value)

    def state(self):
        """(X, Gamma, sigma) of every particle as host arrays."""
        n = self.get_np()
        X, G, S = np.empty((n, 3)), np.empty((n, 3)), np.empty(n)
        L.check(L.lib().vpm_get_state(self._ctx, n, L.dptr(X), 3, L.dptr(G), 3, L.dptr(S), 1),
                self._ctx)
        return X, G, S

    def get_X(self):
        return self.state()[0]

    def get_Gamma(self):
        return self.state()[1]

    def get_sigma(self):
        return self.state()[2]

    def get_UJ(self, i0: int = 0, n: Optional[int] = None):
        """U (n,3) and J (n,3,3) of particles [i0, i0+n) from the last evaluation."""
        if n is None:
            n = self.get_np() - i0
        U, J = np.empty((n, 3)), np.empty((n, 3, 3))
        L.check(L.lib().vpm_get_UJ(self._ctx, i0, n, L.dptr(U), 3, L.dptr(J), 9), self._ctx)
        return U, J

    def get_U(self):
        return self.get_UJ()[0]

    def get_J(self):
        return self.get_UJ()[1]

    def attributes(self):
        """(vol, circulation, static) of every particle as host arrays."""
        n = self.get_np()
        vol, circ = np.empty(n), np.empty(n)
        st = (ctypes.c_int32 * max(n, 1))()
        L.check(L.lib().vpm_get_attributes(self._ctx, 0, n, L.dptr(vol), 1, L.dptr(circ), 1, st),
                self._ctx)
        return vol, circ, np.array(st[:n], dtype=bool)

    def get_vol(self):
        return self.attributes()[0]

    def get_circulation(self):
        return self.attributes()[1]

    def get_static(self):
        return self.attributes()[2]

    def get_C(self):
        n = self.get_np()
        C, E = np.empty((n, 3)), np.empty((n, 3))
        L.check(L.lib().vpm_get_sfs(self._ctx, n, L.dptr(C), 3, L.dptr(E), 3), self._ctx)
        return C

    def get_SFS(self):
        n = self.get_np()
        C, E = np.empty((n, 3)), np.empty((n, 3))
        L.check(L.lib().vpm_get_sfs(self._ctx, n, L.dptr(C), 3, L.dptr(E), 3), self._ctx)
        return E

    @property
    def t(self) -> float:
        t = ctypes.c_double()
        nt = ctypes.c_int64()
        L.check(L.lib().vpm_get_time(self._ctx, ctypes.byref(t), ctypes.byref(nt)), self._ctx)
        return t.value

    @property
    def nt(self) -> int:
        t = ctypes.c_double()
        nt = ctypes.c_int64()
        L.check(L.lib().vpm_get_time(self._ctx, ctypes.byref(t), ctypes.byref(nt)), self._ctx)
        return int(nt.value)

    def eval_UJ_targets(self, t0: int, t1: int, precision: Optional[int] = None):
        """U/J at particles [t0, t1) only (probe evaluation)."""
        self._flush()
        prec = getattr(self.UJ, "precision", L.PREC_FP32C) if precision is None else precision
        L.check(L.lib().vpm_eval_UJ_targets(self._ctx, self.kernel.id, prec, t0, t1), self._ctx)

    def diagnostics(self, precision: Optional[int] = None) -> dict:
        self._flush()
        prec = getattr(self.UJ, "precision", L.PREC_FP32C) if precision is None else precision
        out = np.zeros(L.DIAG_COUNT)
        L.check(L.lib().vpm_diagnostics(self._ctx, self.kernel.id, prec, L.dptr(out)), self._ctx)
        return dict(zip(L.DIAG_NAMES, out.tolist()))

    def centroids(self, ranges):
        self._flush()
        st = (ctypes.c_int64 * len(ranges))(*[r[0] for r in ranges])
        en = (ctypes.c_int64 * len(ranges))(*[r[1] for r in ranges])
        out = np.zeros((len(ranges), 3))
        L.check(L.lib().vpm_centroids(self._ctx, len(ranges), st, en, L.dptr(out)), self._ctx)
        return out


def Ffv_direct(pfield: ParticleField, Xb, Gb, Sb) -> np.ndarray:
    """Free-vortex force terms of bound particles (x_b, Γ_b, σ_b) from every particle
    of the field: columns 0..2 = Σ U_b(x_f) × Γ_f, 3..5 = Σ g_σb K(x_b - x_f) × (Γ_b × Γ_f)
    (_Ffv_direct, src/FLOWUnsteady_processing_force.jl:879-929)."""
    pfield._flush()
    Xb = np.ascontiguousarray(Xb, dtype=np.float64).reshape(-1, 3)
    Gb = np.ascontiguousarray(Gb, dtype=np.float64).reshape(-1, 3)
    Sb = np.ascontiguousarray(Sb, dtype=np.float64).reshape(-1)
    M = np.empty((Xb.shape[0], 6))
    L.check(L.lib().vpm_ffv_direct(pfield._ctx, pfield.kernel.id, Xb.shape[0], L.dptr(Xb), 3,
                                   L.dptr(Gb), 3, L.dptr(Sb), 1, L.dptr(M), 6), pfield._ctx)
    return M


def save(pfield: ParticleField, file_name: str, *, path: str = "", num: Optional[int] = None,
         add_num: bool = True) -> str:
    """Write the particle field (vpm.save, src/FLOWUnsteady_simulation.jl:436-440):
    <path>/<file_name>.pfield[.<num>].xmf and .bin (XDMF + raw FP64, see
    vpm_save).  num defaults to the step counter when add_num; returns the
    .xmf path."""
    pfield._flush()
    if num is None and add_num:
        num = pfield.nt
    prefix = os.path.join(path, file_name) if path else file_name
    L.check(L.lib().vpm_save(pfield._ctx, prefix.encode(), -1 if num is None else int(num)),
            pfield._ctx)
    return prefix + ".pfield" + ("" if num is None else f".{int(num)}") + ".xmf"


def read(pfield: ParticleField, file: str, *, load_time: bool = False):
    """Restore a field written by save (vpm.read!(pfield, file; overwrite=true,
    load_time), src/FLOWUnsteady_simulation.jl:264).  `file` is the .xmf or
    the .bin path."""
    if file.endswith(".xmf"):
        file = file[:-4] + ".bin"
    pfield._pend = []
    L.check(L.lib().vpm_load(pfield._ctx, file.encode(), 1 if load_time else 0), pfield._ctx)
    pfield._uj_valid = False


def add_particle(pfield: ParticleField, X, Gamma, sigma, *, vol=0.0, circulation=1.0, C=None,
                 static: bool = False):
    """Append one particle or an (n,3)/(n,3)/(n,) batch (vpm.add_particle with
    its vol, circulation, C and static keywords)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    G = np.asarray(Gamma, dtype=np.float64).reshape(-1, 3)
    S = np.broadcast_to(np.asarray(sigma, dtype=np.float64).reshape(-1), (n,))
    vol = np.broadcast_to(np.asarray(vol, dtype=np.float64).reshape(-1), (n,))
    circ = np.broadcast_to(np.asarray(circulation, dtype=np.float64).reshape(-1), (n,))
    Cm = (np.zeros((n, 3)) if C is None
          else np.broadcast_to(np.asarray(C, dtype=np.float64).reshape(-1, 3), (n, 3)))
    default = C is None and not np.any(vol != 0.0) and not np.any(circ != 1.0)
    attrs = None if default else (np.array(vol), np.array(circ), np.array(Cm))
    pfield._pend.append((X, G, np.array(S), bool(static), attrs))


def add_probe(pfield: ParticleField, X):
    """Probe particle: a plain particle with Γ = 0, σ = 1e-6 and vol = 0
    (add_probe, src/FLOWUnsteady_simulation.jl:572)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    add_particle(pfield, X, np.zeros_like(X), 1e-6, vol=0.0)


def add_shed_particles(pfield: ParticleField, X, gamma, dt, V, infD, sigma, vol, l,
                       p_per_step: int, *, overwrite_sigma=None, eps: float = 2.0**-52):
    """Shed p_per_step particles along the segment l from X, as FLOWUnsteady's
    add_particle does (src/FLOWUnsteady_simulation.jl:455-489): Γ = γ·(V·dt)·infD,
    raised to 5·eps per component when |Γ| <= 5·eps; circulation max(|γ|, 5·eps);
    each particle carries Γ/p, σ/p (or overwrite_sigma) and vol/p, at
    X + (i - 1/2)·l/p."""
    X = np.asarray(X, dtype=np.float64).reshape(3)
    infD = np.asarray(infD, dtype=np.float64).reshape(3)
    l = np.asarray(l, dtype=np.float64).reshape(3)
    Gamma = gamma * (V * dt) * infD
    if np.sqrt(Gamma @ Gamma) <= 5 * eps:
        Gamma = 5 * eps * np.ones(3)
    circulation = max(abs(gamma), 5 * eps)
    pps = int(p_per_step)
    sigmap = sigma / pps if overwrite_sigma is None else overwrite_sigma
    dX = l / pps
    i = np.arange(1, pps + 1, dtype=np.float64)[:, None]
    add_particle(pfield, X + i * dX - dX / 2, np.tile(Gamma / pps, (pps, 1)), sigmap,
                 vol=vol / pps, circulation=circulation)


def remove_particle(pfield: ParticleField, i: int):
    """Remove particle i (0-based); only the last particle can be removed."""
    n = pfield.get_np()
    if i != n - 1:
        raise ValueError("only tail removal is supported (FLOWUnsteady removes from the tail)")
    L.check(L.lib().vpm_truncate(pfield._ctx, n - 1), pfield._ctx)


def get_np(pfield: ParticleField) -> int:
    return pfield.get_np()


def nextstep(pfield: ParticleField, dt: float, *, relax: bool = False, nsteps: int = 1,
             use_graph: bool = True):
    """Advance the free particles by nsteps steps (vpm.nextstep)."""
    pfield._flush()
    s = pfield.scheme()
    if not relax:
        s.relaxation = L.RELAX_NONE
    L.check(L.lib().vpm_step(pfield._ctx, float(dt), ctypes.byref(s), int(nsteps),
                             1 if use_graph else 0), pfield._ctx)


def Vvpm_on_Xs(pfield: ParticleField, Xs) -> np.ndarray:
    """Velocity of the field at points Xs: probes appended, U/J evaluated at the
    probes only, probes removed (Vvpm_on_Xs, src/FLOWUnsteady_simulation.jl:494-570)."""
    Xs = np.asarray(Xs, dtype=np.float64).reshape(-1, 3)
    if Xs.shape[0] == 0:
        return np.zeros((0, 3))
    n0 = pfield.get_np()
    add_probe(pfield, Xs)
    pfield.eval_UJ_targets(n0, n0 + Xs.shape[0])
    U, _ = pfield.get_UJ(n0, Xs.shape[0])
    L.check(L.lib().vpm_truncate(pfield._ctx, n0), pfield._ctx)
    return U


def monitor_enstrophy(pfield: ParticleField) -> float:
    """½ Σ Γ_p·ω(x_p) (src/FLOWUnsteady_monitors.jl:573-574)."""
    return pfield.diagnostics()["enstrophy"]


def monitor_Cd(pfield: ParticleField) -> dict:
    """Statistics of the SFS coefficient over the free particles, in the order of
    vpm.monitor_Cd's record (src/FLOWUnsteady_monitors.jl:697-703): t, ratio of
    zeros, then mean, standard deviation, skewness, excess kurtosis, minimum and
    maximum of the nonzero C_d."""
    d = pfield.diagnostics()
    return {"t": pfield.t, "cd_zero_ratio": d["cd_zero_ratio"], "cd_mean": d["cd_mean"],
            "cd_std": d["cd_std"], "cd_skew": d["cd_skew"], "cd_kurt": d["cd_kurt"],
            "cd_min": d["cd_min"], "cd_max": d["cd_max"]}


def measure_fma_peaks(device: int = 0):
    f32, f64, mhz = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    L.check(L.lib().vpm_measure_fma_peaks(device, ctypes.byref(f32), ctypes.byref(f64),
                                          ctypes.byref(mhz)))
    return f32.value, f64.value, mhz.value

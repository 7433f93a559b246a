"""Python binding of the engine's C ABI (include/komd_gpu.h) via ctypes.

The engine is the in-tree shared library komd_gb300/_build/libkomd_gpu.so;
there is no Python or CPU fallback: if the library is missing or cannot be
loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Dict, List, Optional

import numpy as np

from .build import LIB_GPU

KOMD_OK = 0
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_OVERFLOW", 4: "ERR_STATE", 5: "ERR_NOMEM", 6: "ERR_NONFINITE"}

FP32, FP64 = 0, 1
ATM_SIGN_REFERENCE, ATM_SIGN_PHYSICAL = 0, 1
ATM_ENUM_COMPAT, ATM_ENUM_FULL = 0, 1
VIRIAL_COMPAT, VIRIAL_CORRECT = 0, 1

TERM_LJ, TERM_FENE, TERM_LIMIT, TERM_ATM, TERM_BONDED, TERM_ATM_SURROGATE = 0x01, 0x02, 0x04, 0x08, 0x10, 0x20
TERM_ATM2B, TERM_TABULATED = 0x40, 0x80
SUR_NFEAT, SUR_NPARAM = 32, 6337
FIT_BF16, FIT_FP32 = 0, 1
MEASURE_TEMPERATURE, MEASURE_ENERGY, MEASURE_PRESSURE, MEASURE_RDF, MEASURE_LJ_HIST = 0x01, 0x02, 0x04, 0x08, 0x10

EXPORTS = [
    "komd_gpu_create", "komd_gpu_destroy", "komd_gpu_last_error", "komd_gpu_abi_version", "komd_gpu_set_stream",
    "komd_sci_temperature", "komd_batch_measure",
    "komd_gpu_grid_dims", "komd_gpu_upload_sites", "komd_gpu_set_state", "komd_gpu_set_topology",
    "komd_gpu_download", "komd_gpu_num_sites", "komd_gpu_update_container", "komd_gpu_forces",
    "komd_gpu_integrate0", "komd_gpu_integrate1", "komd_gpu_step", "komd_gpu_step_host", "komd_gpu_measure",
    "komd_gpu_rdf_bins", "komd_gpu_get_cells", "komd_gpu_neighbour_counts", "komd_gpu_set_profiling",
    "komd_gpu_profile", "komd_gpu_kernels_per_step", "komd_gpu_atm_forces_noalloc", "komd_gpu_surrogate_load",
    "komd_gpu_surrogate_sample", "komd_gpu_surrogate_forces", "komd_gpu_surrogate_status", "komd_mlp_train",
    "komd_mlp_loss_grad", "komd_sur_data_create", "komd_sur_data_destroy", "komd_gpu_surrogate_capture",
    "komd_sur_data_snapshots", "komd_sur_data_sites", "komd_sur_data_get", "komd_sur_fit", "komd_sur_fit_grad",
    "komd_gpu_scale_velocities", "komd_gpu_set_pair_table", "komd_gpu_rdf_profile", "komd_gpu_set_terms", "komd_batch_create", "komd_batch_destroy", "komd_batch_step", "komd_batch_launch", "komd_batch_check",
    "komd_batch_form",
]


class KomdConfig(C.Structure):
    _fields_ = [
        ("domain_low", C.c_double * 3), ("domain_high", C.c_double * 3), ("cell_size", C.c_double),
        ("cutoff", C.c_double), ("cutoff_3b", C.c_double), ("nu", C.c_double), ("delta_t", C.c_double),
        ("stiffness", C.c_double), ("limit", C.c_double), ("bond_k", C.c_double), ("bond_r0", C.c_double),
        ("angle_k", C.c_double), ("angle_theta0", C.c_double), ("max_sigma", C.c_double), ("rdf_max", C.c_double),
        ("rdf_dr", C.c_double), ("terms", C.c_uint32), ("precision", C.c_int32), ("atm_sign", C.c_int32),
        ("atm_enum", C.c_int32), ("virial_mode", C.c_int32), ("atm_direct", C.c_int32), ("lj_bins", C.c_int32),
        ("atm_list_cap", C.c_int32), ("skin", C.c_double), ("temperature_target", C.c_double),
        ("thermostat", C.c_int32), ("switch_width", C.c_double),
    ]


class Observables(C.Structure):
    _fields_ = [
        ("temperature", C.c_double), ("mv2", C.c_double), ("n_in_box", C.c_double), ("u_lj", C.c_double),
        ("u_atm", C.c_double), ("u_bonded", C.c_double), ("kinetic", C.c_double * 6), ("virial", C.c_double * 6),
        ("pressure", C.c_double * 6), ("pairs_in_cutoff", C.c_int64), ("triplets", C.c_int64),
    ]


class SurrogateStatus(C.Structure):
    _fields_ = [("steps", C.c_int64), ("probes", C.c_int64), ("last_rmse", C.c_double), ("max_rmse", C.c_double),
                ("fallback", C.c_int32), ("fallback_step", C.c_int64)]


class SurFitOpts(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("snaps_per_batch", C.c_int32), ("lr", C.c_float), ("lr_end", C.c_float),
                ("lam_e", C.c_float), ("lam_f", C.c_float), ("seed", C.c_uint64), ("precision", C.c_int32)]


class KomdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"komd_gpu {STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    return LIB_GPU


def load() -> C.CDLL:
    """Loads the native engine; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_GPU):
        raise RuntimeError(f"native engine {LIB_GPU} is not built: run `python -m komd_gb300.build` first "
                           "(there is no CPU fallback)")
    L = C.CDLL(LIB_GPU)
    P, I64, I32 = C.c_void_p, C.c_int64, C.c_int
    L.komd_gpu_create.argtypes = [C.POINTER(KomdConfig), I32, C.POINTER(P)]
    L.komd_gpu_destroy.argtypes = [P]
    L.komd_gpu_last_error.restype = C.c_char_p
    L.komd_sci_temperature.argtypes = [C.c_double, C.c_double]
    L.komd_sci_temperature.restype = C.c_double
    L.komd_gpu_set_stream.argtypes = [P, P]
    L.komd_gpu_grid_dims.argtypes = [P, P]
    L.komd_gpu_upload_sites.argtypes = [P, I64, P, P, P, P, P, P]
    L.komd_gpu_set_state.argtypes = [P, P, P]
    L.komd_gpu_set_topology.argtypes = [P, I64, P, I64, P]
    L.komd_gpu_download.argtypes = [P, P, P, P]
    L.komd_gpu_num_sites.argtypes = [P]
    L.komd_gpu_num_sites.restype = I64
    for fn in ("komd_gpu_update_container", "komd_gpu_forces", "komd_gpu_integrate0", "komd_gpu_integrate1"):
        getattr(L, fn).argtypes = [P]
    L.komd_gpu_step.argtypes = [P, I64]
    L.komd_gpu_step_host.argtypes = [P, I64, P, P, P]
    L.komd_gpu_measure.argtypes = [P, C.c_uint32, C.POINTER(Observables), P, P]
    L.komd_gpu_rdf_bins.argtypes = [P]
    L.komd_gpu_rdf_bins.restype = I64
    L.komd_gpu_get_cells.argtypes = [P, P, I64, P, I64, C.POINTER(I64)]
    L.komd_gpu_neighbour_counts.argtypes = [P, P]
    L.komd_gpu_set_profiling.argtypes = [P, I32]
    L.komd_gpu_profile.argtypes = [P, I32, P, P, C.c_char_p, I32]
    L.komd_gpu_kernels_per_step.argtypes = [P]
    L.komd_gpu_atm_forces_noalloc.argtypes = [I64, P, P, P, P, C.c_double, C.c_double, C.c_int32, P]
    L.komd_gpu_surrogate_load.argtypes = [P, P, P, P, C.c_double, C.c_double, C.c_int32, C.c_double]
    L.komd_gpu_surrogate_sample.argtypes = [P, P, P, P]
    L.komd_gpu_surrogate_forces.argtypes = [P, P, P]
    L.komd_gpu_surrogate_status.argtypes = [P, C.POINTER(SurrogateStatus)]
    L.komd_mlp_train.argtypes = [P, P, I64, P, C.c_int32, C.c_int32, C.c_float, C.c_uint64, P]
    L.komd_mlp_loss_grad.argtypes = [P, P, I64, P, P, P]
    L.komd_sur_data_create.argtypes = [I32, I32, C.POINTER(P)]
    L.komd_sur_data_destroy.argtypes = [P]
    L.komd_sur_data_destroy.restype = None
    L.komd_gpu_surrogate_capture.argtypes = [P, P]
    L.komd_sur_data_snapshots.argtypes = [P]
    L.komd_sur_data_snapshots.restype = I64
    L.komd_sur_data_sites.argtypes = [P]
    L.komd_sur_data_get.argtypes = [P, I64, P, P, P, P]
    L.komd_sur_fit.argtypes = [P, P, P, P, C.c_double, C.c_double, C.c_double, C.POINTER(SurFitOpts), P]
    L.komd_gpu_scale_velocities.argtypes = [P, C.c_double]
    L.komd_gpu_set_pair_table.argtypes = [P, I32, P, P, C.c_double, C.c_double]
    L.komd_gpu_rdf_profile.argtypes = [P, C.c_double, I32, P]
    L.komd_gpu_set_terms.argtypes = [P, C.c_uint32]
    L.komd_batch_create.argtypes = [P, I32, I32, I32, P, C.POINTER(P)]
    L.komd_batch_destroy.argtypes = [P]
    L.komd_batch_destroy.restype = None
    L.komd_batch_step.argtypes = [P, I64]
    L.komd_batch_launch.argtypes = [P, I64]
    L.komd_batch_check.argtypes = [P]
    L.komd_batch_form.argtypes = [P]
    L.komd_batch_measure.argtypes = [P, C.c_uint32, P, P]
    L.komd_sur_fit_grad.argtypes = [P, P, P, P, C.c_double, C.c_double, C.c_double, C.c_float, C.c_float, P, P,
                                    C.c_int32]
    _lib = L
    return L


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def make_config(low, high, cell_size, cutoff=2.5, cutoff_3b=None, nu=0.0, dt=0.005, terms=TERM_LJ,
                precision=FP32, atm_sign=ATM_SIGN_REFERENCE, atm_enum=ATM_ENUM_COMPAT, virial_mode=VIRIAL_COMPAT,
                atm_direct=1, stiffness=30.0, limit=1e30, bond_k=0.0, bond_r0=1.0, angle_k=0.0, angle_theta0=0.0,
                max_sigma=1.0, rdf_max=0.0, rdf_dr=0.0, lj_bins=100, atm_list_cap=0, skin=0.0,
                thermostat=0, temperature_target=0.0, switch_width=0.0) -> KomdConfig:
    c = KomdConfig()
    for d in range(3):
        c.domain_low[d] = float(low[d])
        c.domain_high[d] = float(high[d])
    c.cell_size = float(cell_size)
    c.cutoff = float(cutoff)
    c.cutoff_3b = float(cutoff if cutoff_3b is None else cutoff_3b)
    c.nu, c.delta_t, c.stiffness, c.limit = float(nu), float(dt), float(stiffness), float(limit)
    c.bond_k, c.bond_r0, c.angle_k, c.angle_theta0 = float(bond_k), float(bond_r0), float(angle_k), float(angle_theta0)
    c.max_sigma, c.rdf_max, c.rdf_dr = float(max_sigma), float(rdf_max), float(rdf_dr)
    c.terms, c.precision, c.atm_sign, c.atm_enum = int(terms), int(precision), int(atm_sign), int(atm_enum)
    c.virial_mode, c.atm_direct, c.lj_bins, c.atm_list_cap = int(virial_mode), int(atm_direct), int(lj_bins), int(atm_list_cap)
    c.skin = float(skin)
    c.thermostat, c.temperature_target = int(thermostat), float(temperature_target)
    c.switch_width = float(switch_width)
    return c


class GpuSystem:
    """One periodic system on one GPU behind the C ABI."""

    def __init__(self, sysm, cfg: KomdConfig, device: int = 0):
        self.L = load()
        self.h = C.c_void_p()
        self._check(self.L.komd_gpu_create(C.byref(cfg), int(device), C.byref(self.h)))
        self.cfg = cfg
        self.n = int(sysm.n)
        r = np.ascontiguousarray(sysm.r, np.float64)
        v = np.ascontiguousarray(sysm.v, np.float64)
        self._keep = [np.ascontiguousarray(x, np.float64) for x in (sysm.m, sysm.eps, sysm.sig)]
        mid = np.ascontiguousarray(sysm.mol_id, np.uint64)
        self._check(self.L.komd_gpu_upload_sites(self.h, self.n, _p(r), _p(v), _p(self._keep[0]), _p(self._keep[1]),
                                                 _p(self._keep[2]), _p(mid)))
        bonds = getattr(sysm, "bonds", None)
        angles = getattr(sysm, "angles", None)
        if (bonds is not None and len(bonds)) or (angles is not None and len(angles)):
            b = np.ascontiguousarray(bonds if bonds is not None else np.zeros((0, 2)), np.int64)
            a = np.ascontiguousarray(angles if angles is not None else np.zeros((0, 3)), np.int64)
            self._check(self.L.komd_gpu_set_topology(self.h, b.shape[0], _p(b), a.shape[0], _p(a)))

    def _check(self, code):
        if code != KOMD_OK:
            raise KomdError(code, self.L.komd_gpu_last_error().decode())

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.komd_gpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- hot path ---------------------------------------------------------
    def update_container(self):
        self._check(self.L.komd_gpu_update_container(self.h))

    def forces(self):
        self._check(self.L.komd_gpu_forces(self.h))

    def integrate0(self):
        self._check(self.L.komd_gpu_integrate0(self.h))

    def integrate1(self):
        self._check(self.L.komd_gpu_integrate1(self.h))

    def step(self, n: int = 1):
        self._check(self.L.komd_gpu_step(self.h, int(n)))

    def step_host(self, n, r, v, f):
        self._check(self.L.komd_gpu_step_host(self.h, int(n), _p(r), _p(v), _p(f)))

    def set_state(self, r=None, v=None):
        r = None if r is None else np.ascontiguousarray(r, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        self._check(self.L.komd_gpu_set_state(self.h, _p(r), _p(v)))

    def set_stream(self, stream_ptr: int):
        self._check(self.L.komd_gpu_set_stream(self.h, C.c_void_p(stream_ptr)))

    def download(self):
        r = np.empty((self.n, 3))
        v = np.empty((self.n, 3))
        f = np.empty((self.n, 3))
        self._check(self.L.komd_gpu_download(self.h, _p(r), _p(v), _p(f)))
        return r, v, f

    # --- sensors ----------------------------------------------------------
    def measure(self, mask: int) -> Dict[str, object]:
        obs = Observables()
        nb = int(self.L.komd_gpu_rdf_bins(self.h))
        rdf = np.zeros(max(nb, 1))
        hist = np.zeros(4 * self.cfg.lj_bins)
        self._check(self.L.komd_gpu_measure(self.h, int(mask), C.byref(obs), _p(rdf), _p(hist)))
        out = {k: getattr(obs, k) for k, _ in Observables._fields_}
        for k in ("kinetic", "virial", "pressure"):
            out[k] = np.array(out[k][:])
        out["rdf"] = rdf[:nb] if nb > 0 else None
        out["lj_hist"] = hist.reshape(4, -1)
        return out

    # --- parity dumps -----------------------------------------------------
    def grid_dims(self):
        nd = np.zeros(3, np.int64)
        self._check(self.L.komd_gpu_grid_dims(self.h, _p(nd)))
        return tuple(int(x) for x in nd)

    def cells(self):
        nd = self.grid_dims()
        ncell = (nd[0] + 2) * (nd[1] + 2) * (nd[2] + 2)
        count = np.zeros(ncell, np.int64)
        total = C.c_int64(0)
        self._check(self.L.komd_gpu_get_cells(self.h, _p(count), ncell, None, 0, C.byref(total)))
        idx = np.zeros(max(total.value, 1), np.int64)
        self._check(self.L.komd_gpu_get_cells(self.h, _p(count), ncell, _p(idx), total.value, C.byref(total)))
        return count, idx[:total.value]

    def neighbour_counts(self):
        c = np.zeros(self.n, np.int64)
        self._check(self.L.komd_gpu_neighbour_counts(self.h, _p(c)))
        return c

    # --- profiling --------------------------------------------------------
    def set_profiling(self, on: bool):
        self._check(self.L.komd_gpu_set_profiling(self.h, 1 if on else 0))

    def profile(self):
        launches = np.zeros(16, np.int64)
        ms = np.zeros(16)
        names = C.create_string_buffer(512)
        nf = self.L.komd_gpu_profile(self.h, 16, _p(launches), _p(ms), names, 512)
        if nf < 0:
            self._check(nf)
        fams = names.value.decode().split("\n")[:nf]
        return {f: (int(launches[i]), float(ms[i])) for i, f in enumerate(fams)}

    def kernels_per_step(self) -> int:
        return int(self.L.komd_gpu_kernels_per_step(self.h))

    # --- learned three-body term ------------------------------------------
    def surrogate_load(self, model, probe_every=50, probe_threshold=0.05):
        p = np.ascontiguousarray(model["params"], np.float32)
        fm = np.ascontiguousarray(model["fmean"], np.float32)
        fs = np.ascontiguousarray(model["fstd"], np.float32)
        self._sur_keep = (p, fm, fs)
        self._check(self.L.komd_gpu_surrogate_load(self.h, _p(p), _p(fm), _p(fs), float(model["e_scale"]),
                                                   float(model["e_shift"]), int(probe_every), float(probe_threshold)))

    def surrogate_sample(self):
        x = np.zeros((self.n, SUR_NFEAT), np.float32)
        e3 = np.zeros(self.n)
        f3 = np.zeros((self.n, 3))
        self._check(self.L.komd_gpu_surrogate_sample(self.h, _p(x), _p(e3), _p(f3)))
        return x, e3, f3

    def scale_velocities(self, beta: float):
        """VelocityScaling::apply with the caller's beta (v *= beta)."""
        self._check(self.L.komd_gpu_scale_velocities(self.h, float(beta)))

    def set_pair_table(self, x, y, below=1e6, above=0.0):
        """Tabulated pair force F(r) (KOMD_TERM_TABULATED), piecewise linear."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        self._check(self.L.komd_gpu_set_pair_table(self.h, x.size, _p(x), _p(y), float(below), float(above)))

    def set_terms(self, terms: int):
        """Replaces the step's force terms (a plugin swapping the functors)."""
        self._check(self.L.komd_gpu_set_terms(self.h, int(terms)))

    def rdf_profile(self, max_r, nbins):
        """RDF_Profiler histogram (ordered COM pairs, nbins bins up to max_r)."""
        b = np.zeros(int(nbins))
        self._check(self.L.komd_gpu_rdf_profile(self.h, float(max_r), int(nbins), _p(b)))
        return b

    def surrogate_capture(self, data: "SurData"):
        """Appends the current state to a force-matching dataset."""
        self._check(self.L.komd_gpu_surrogate_capture(self.h, data.h))

    def surrogate_forces(self):
        f3 = np.zeros((self.n, 3))
        e3 = np.zeros(self.n)
        self._check(self.L.komd_gpu_surrogate_forces(self.h, _p(f3), _p(e3)))
        return f3, e3

    def surrogate_status(self):
        st = SurrogateStatus()
        self._check(self.L.komd_gpu_surrogate_status(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in SurrogateStatus._fields_}


def mlp_train(X, y, params, epochs, batch=1024, lr=2e-3, seed=0):
    L = load()
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    p = np.ascontiguousarray(params, np.float32).copy()
    loss = np.zeros(max(epochs, 1), np.float32)
    rc = L.komd_mlp_train(_p(X), _p(y), X.shape[0], _p(p), int(epochs), int(batch), float(lr), int(seed), _p(loss))
    if rc != KOMD_OK:
        raise KomdError(rc, L.komd_gpu_last_error().decode())
    return p, loss[:epochs]


def mlp_loss_grad(X, y, params):
    L = load()
    X = np.ascontiguousarray(X, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    p = np.ascontiguousarray(params, np.float32)
    g = np.zeros(SUR_NPARAM, np.float32)
    loss = np.zeros(1, np.float32)
    rc = L.komd_mlp_loss_grad(_p(X), _p(y), X.shape[0], _p(p), _p(g), _p(loss))
    if rc != KOMD_OK:
        raise KomdError(rc, L.komd_gpu_last_error().decode())
    return g, float(loss[0])


class SurData:
    """Snapshots for force-matched training, resident on the device."""

    def __init__(self, device=0, nl_cap=80):
        self.L = load()
        self.h = C.c_void_p()
        rc = self.L.komd_sur_data_create(int(device), int(nl_cap), C.byref(self.h))
        if rc != KOMD_OK:
            raise KomdError(rc, self.L.komd_gpu_last_error().decode())

    def _check(self, rc):
        if rc != KOMD_OK:
            raise KomdError(rc, self.L.komd_gpu_last_error().decode())

    @property
    def snapshots(self) -> int:
        return int(self.L.komd_sur_data_snapshots(self.h))

    @property
    def sites(self) -> int:
        return int(self.L.komd_sur_data_sites(self.h))

    def get(self, snap=-1):
        """(features, e3, f3, site) of one snapshot or of all (snap < 0), slot order."""
        n = self.sites * (self.snapshots if snap < 0 else 1)
        x = np.zeros((n, SUR_NFEAT), np.float32)
        e3 = np.zeros(n, np.float32)
        f3 = np.zeros((n, 3), np.float32)
        site = np.zeros(n, np.int32)
        self._check(self.L.komd_sur_data_get(self.h, int(snap), _p(x), _p(e3), _p(f3), _p(site)))
        return x, e3, f3, site

    def fit(self, params, fmean, fstd, e_scale, e_shift, f2, epochs, snaps_per_batch=4, lr=2e-3, lr_end=1e-4,
            lam_e=0.1, lam_f=1.0, seed=0, precision=FIT_BF16):
        o = SurFitOpts(int(epochs), int(snaps_per_batch), float(lr), float(lr_end), float(lam_e), float(lam_f),
                       int(seed), int(precision))
        p = np.ascontiguousarray(params, np.float32).copy()
        fm = np.ascontiguousarray(fmean, np.float32)
        fs = np.ascontiguousarray(fstd, np.float32)
        loss = np.zeros(2 * max(int(epochs), 1), np.float32)
        self._check(self.L.komd_sur_fit(self.h, _p(p), _p(fm), _p(fs), float(e_scale), float(e_shift), float(f2),
                                        C.byref(o), _p(loss)))
        return p, loss[:2 * int(epochs)].reshape(-1, 2)

    def fit_grad(self, params, fmean, fstd, e_scale, e_shift, f2, lam_e=0.1, lam_f=1.0, precision=FIT_BF16):
        p = np.ascontiguousarray(params, np.float32)
        fm = np.ascontiguousarray(fmean, np.float32)
        fs = np.ascontiguousarray(fstd, np.float32)
        g = np.zeros(SUR_NPARAM, np.float32)
        loss = np.zeros(2)
        self._check(self.L.komd_sur_fit_grad(self.h, _p(p), _p(fm), _p(fs), float(e_scale), float(e_shift), float(f2),
                                             float(lam_e), float(lam_f), _p(g), _p(loss), int(precision)))
        return g, loss

    def close(self):
        if self.h:
            self.L.komd_sur_data_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Replicas (GpuSystem objects, each past update_container + forces)
    advanced together by one CUDA graph of steps_per_graph steps each."""

    def __init__(self, systems, n_streams=16, steps_per_graph=1, stream=None):
        self.L = load()
        self.systems = list(systems)
        arr = (C.c_void_p * len(self.systems))(*[g.h.value if isinstance(g.h, C.c_void_p) else g.h
                                                 for g in self.systems])
        self.h = C.c_void_p()
        self.steps_per_graph = int(steps_per_graph)
        rc = self.L.komd_batch_create(arr, len(self.systems), int(n_streams), self.steps_per_graph, stream,
                                      C.byref(self.h))
        if rc != KOMD_OK:
            raise KomdError(rc, self.L.komd_gpu_last_error().decode())

    def _check(self, rc):
        if rc != KOMD_OK:
            raise KomdError(rc, self.L.komd_gpu_last_error().decode())

    def step(self, n_graphs=1):
        self._check(self.L.komd_batch_step(self.h, int(n_graphs)))

    def launch(self, n_graphs=1):
        self._check(self.L.komd_batch_launch(self.h, int(n_graphs)))

    @property
    def packed(self) -> bool:
        """True when one launch per stage advances every replica (komd_batch_form)."""
        return int(self.L.komd_batch_form(self.h)) == 1

    def check(self):
        self._check(self.L.komd_batch_check(self.h))

    def measure(self, mask: int) -> List[Dict[str, object]]:
        """Every replica's observables (komd_batch_measure), one dict per
        replica as GpuSystem.measure gives it (no LJ histograms)."""
        n = len(self.systems)
        obs = (Observables * n)()
        bins = [int(self.L.komd_gpu_rdf_bins(g.h)) if mask & MEASURE_RDF else 0 for g in self.systems]
        rdf = np.zeros(max(sum(bins), 1))
        self._check(self.L.komd_batch_measure(self.h, int(mask), C.cast(obs, C.c_void_p), _p(rdf)))
        out, off = [], 0
        for k in range(n):
            d = {f: getattr(obs[k], f) for f, _ in Observables._fields_}
            for f in ("kinetic", "virial", "pressure"):
                d[f] = np.array(d[f][:])
            d["rdf"] = rdf[off:off + bins[k]].copy() if bins[k] > 0 else None
            off += bins[k]
            out.append(d)
        return out

    def close(self):
        if self.h:
            self.L.komd_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

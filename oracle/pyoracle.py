"""ctypes binding of the FP64 CPU oracle (oracle/komd_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg -- never by the engine in komd_gb300/.

`OracleSim` restates one reference MD step (Simulation.cpp:49-74 without the
thermostat) on numpy arrays:

    integrate0 -> update_container (COM, wrap, f = 0, COM, bin)
               -> LJ (+ FENE) (+ Limit) (+ ATM) -> integrate1
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libkomd_oracle.so")

P = C.c_void_p
I64 = C.c_int64
D = C.c_double

VIRIAL_COMPAT, VIRIAL_CORRECT = 0, 1
ATM_SIGN_REFERENCE, ATM_SIGN_PHYSICAL = 0, 1


class Grid(C.Structure):
    _fields_ = [("low", D * 3), ("high", D * 3), ("L", D * 3), ("cs", D), ("nd", I64 * 3), ("nc", I64 * 3),
                ("ncell", I64), ("bl", P * 3), ("bh", P * 3)]


class Cells(C.Structure):
    _fields_ = [("ncell", I64), ("count", C.POINTER(I64)), ("start", C.POINTER(I64)), ("idx", C.POINTER(I64)),
                ("total", I64)]


class LJOut(C.Structure):
    _fields_ = [("u_total", D), ("virial", D * 6), ("pairs_in_cutoff", I64)]


class ATMOut(C.Structure):
    _fields_ = [("energy", D), ("virial", D * 6), ("triplets", I64)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.kor_grid_init.argtypes = [C.POINTER(Grid), P, P, D]
        L.kor_grid_free.argtypes = [C.POINTER(Grid)]
        L.kor_com.argtypes = [I64, P, P, P, P]
        L.kor_wrap.argtypes = [C.POINTER(Grid), I64, P, P, P]
        L.kor_bin.argtypes = [C.POINTER(Grid), I64, P, P, C.POINTER(Cells)]
        L.kor_cells_free.argtypes = [C.POINTER(Cells)]
        L.kor_c08_pairs.argtypes = [C.POINTER(Grid), I64, P, P]
        L.kor_c08_pairs.restype = I64
        L.kor_c08_triples.argtypes = [C.POINTER(Grid), I64, P, P]
        L.kor_c08_triples.restype = I64
        L.kor_pair_list.argtypes = [C.POINTER(Grid), C.POINTER(Cells), I64, P, P]
        L.kor_pair_list.restype = I64
        L.kor_lj.argtypes = [C.POINTER(Grid), I64, P, P, P, P, P, P, D, C.c_int, P, P, C.POINTER(LJOut), I64, D, P, P, P, P]
        L.kor_lj_cells.argtypes = [C.POINTER(Grid), C.POINTER(Cells), P, P, P, P, D, P, C.POINTER(LJOut)]
        L.kor_atm_compat.argtypes = [C.POINTER(Grid), C.POINTER(Cells), P, D, D, C.c_int, C.c_int, C.c_int, P,
                                     C.POINTER(ATMOut)]
        L.kor_atm_vertex.argtypes = [C.POINTER(Grid), C.POINTER(Cells), P, D, D, C.c_int, C.c_int, P, C.POINTER(ATMOut)]
        L.kor_atm_comp_force.argtypes = [D, D, D, D]
        L.kor_atm_comp_force.restype = D
        L.kor_atm_energy.argtypes = [D, D, D, D]
        L.kor_atm_energy.restype = D
        L.kor_fene.argtypes = [I64, P, P, P, P, P, P, D, P]
        L.kor_limit.argtypes = [I64, P, P, D, P]
        L.kor_bonded.argtypes = [I64, P, D, D, I64, P, D, D, P, P, P, P]
        L.kor_bonded.restype = D
        L.kor_step0.argtypes = [I64, P, P, P, P, D]
        L.kor_step1.argtypes = [I64, P, P, P, D]
        L.kor_temperature.argtypes = [I64, P, P, P, P, P]
        L.kor_pair_table.argtypes = [I64, P, P, P, D, I64, P, P, D, D, P]
        L.kor_pair_table.restype = None
        L.kor_set_lj_force_scale.argtypes = [D]
        L.kor_set_lj_force_scale.restype = None
        L.kor_set_switch.argtypes = [D, D]
        L.kor_set_switch.restype = None
        L.kor_atm2b_factor.argtypes = [D, D, D, D, D]
        L.kor_atm2b_factor.restype = D
        L.kor_temperature.restype = D
        L.kor_momentum.argtypes = [I64, P, P, P]
        L.kor_rdf_nbins.argtypes = [D, D]
        L.kor_rdf_nbins.restype = I64
        L.kor_rdf.argtypes = [I64, P, P, D, D, I64, P]
        L.kor_pressure_factor.restype = D
        L.kor_num_threads.restype = C.c_int
        L.kor_set_num_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n: int) -> None:
    lib().kor_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().kor_num_threads())


class OracleSim:
    """Owns copies of the site arrays and runs reference-semantics steps."""

    def __init__(self, sysm, cell_size, cutoff, dt=0.005, nu=0.0, cutoff_atm=None, limit=1e30,
                 stiffness=30.0, lj=True, atm=False, atm_mode="compat", atm_sign=ATM_SIGN_REFERENCE,
                 fene=False, bonded=None, virial_mode=VIRIAL_COMPAT, lj_force_scale=1.0, table=None,
                 switch_width=0.0):
        self.L = lib()
        self.r = np.ascontiguousarray(sysm.r, dtype=np.float64).copy()
        self.v = np.ascontiguousarray(sysm.v, dtype=np.float64).copy()
        self.f = np.zeros_like(self.r)
        self.m = np.ascontiguousarray(sysm.m, dtype=np.float64)
        self.eps = np.ascontiguousarray(sysm.eps, dtype=np.float64)
        self.sig = np.ascontiguousarray(sysm.sig, dtype=np.float64)
        self.id = np.ascontiguousarray(sysm.mol_id, dtype=np.uint64)
        self.mol_off = np.ascontiguousarray(sysm.mol_off, dtype=np.int64)
        self.n = self.r.shape[0]
        self.n_mol = self.mol_off.shape[0] - 1
        self.com = np.zeros((self.n_mol, 3))
        self.low = np.ascontiguousarray(sysm.low, dtype=np.float64)
        self.high = np.ascontiguousarray(sysm.high, dtype=np.float64)
        self.g = Grid()
        if self.L.kor_grid_init(C.byref(self.g), _p(self.low), _p(self.high), float(cell_size)) != 0:
            raise ValueError("domain smaller than one cell")
        self.cells = Cells()
        self.cutoff, self.cutoff_atm = float(cutoff), float(cutoff if cutoff_atm is None else cutoff_atm)
        self.dt, self.nu, self.limit, self.stiffness = float(dt), float(nu), float(limit), float(stiffness)
        self.use_lj, self.use_atm, self.use_fene = lj, atm, fene
        self.atm_mode, self.atm_sign, self.virial_mode = atm_mode, atm_sign, virial_mode
        self.bonded = bonded
        self.lj_force_scale = float(lj_force_scale)   # ATM2B potential_factor (1 = LJ12_6)
        # the switched-cutoff option (kor_set_switch): width of the switch below
        # each cutoff, 0 = the reference's truncated potentials
        self.switch_width = float(switch_width)
        # tabulated pair force (x, y, below, above) in place of / after LJ
        self.table = None if table is None else (np.ascontiguousarray(table[0], np.float64),
                                                 np.ascontiguousarray(table[1], np.float64),
                                                 float(table[2]), float(table[3]))
        self.lj_out, self.atm_out = LJOut(), ATMOut()
        self.e_bonded = 0.0
        self.ncount = None

    def __del__(self):
        try:
            self.L.kor_cells_free(C.byref(self.cells))
            self.L.kor_grid_free(C.byref(self.g))
        except Exception:
            pass

    # --- container -------------------------------------------------------
    def update_container(self):
        L = self.L
        L.kor_com(self.n_mol, _p(self.mol_off), _p(self.r), _p(self.m), _p(self.com))
        L.kor_wrap(C.byref(self.g), self.n_mol, _p(self.mol_off), _p(self.com), _p(self.r))
        self.f[:] = 0
        L.kor_com(self.n_mol, _p(self.mol_off), _p(self.r), _p(self.m), _p(self.com))
        L.kor_bin(C.byref(self.g), self.n_mol, _p(self.mol_off), _p(self.com), C.byref(self.cells))

    def cell_lists(self):
        """(count, start, idx) of the reference's (nd+2)^3 grid incl. halo copies."""
        c = self.cells
        count = np.ctypeslib.as_array(c.count, shape=(c.ncell,)).copy()
        start = np.ctypeslib.as_array(c.start, shape=(c.ncell + 1,)).copy()
        idx = np.ctypeslib.as_array(c.idx, shape=(max(c.total, 1),))[:c.total].copy()
        return count, start, idx

    @property
    def nd(self):
        return tuple(int(x) for x in self.g.nd)

    def pair_list(self):
        n = self.L.kor_pair_list(C.byref(self.g), C.byref(self.cells), 0, None, None)
        pairs = np.zeros((max(n, 1), 2), np.int64)
        shifts = np.zeros((max(n, 1), 6), np.float64)
        self.L.kor_pair_list(C.byref(self.g), C.byref(self.cells), n, _p(pairs), _p(shifts))
        return pairs[:n], shifts[:n]

    # --- forces ------------------------------------------------------------
    def forces(self, nbins=0, max_sigma=1.0, with_atm_virial=False, ncount=False, listless=False):
        self.L.kor_set_lj_force_scale(self.lj_force_scale)
        self.L.kor_set_switch(self.switch_width, self.switch_width)
        try:
            self._forces(nbins, max_sigma, with_atm_virial, ncount, listless)
        finally:
            self.L.kor_set_lj_force_scale(1.0)
            self.L.kor_set_switch(0.0, 0.0)

    def thermostat(self, t_target):
        """VelocityScaling::apply (VelocityScaling.cpp:12-25) after a
        temperature measure: v *= sqrt(T_target / T)."""
        beta = np.sqrt(t_target / self.temperature())
        self.v *= beta
        return beta

    def _forces(self, nbins, max_sigma, with_atm_virial, ncount, listless):
        if listless:
            # large systems: LJ straight from the cells, no materialised pair list
            if self.use_fene or nbins or ncount:
                raise ValueError("listless forces cover LJ, the bonded terms, Limit and ATM only")
            if self.use_lj:
                self.L.kor_lj_cells(C.byref(self.g), C.byref(self.cells), _p(self.r), _p(self.eps), _p(self.sig),
                                    _p(self.id), self.cutoff, _p(self.f), C.byref(self.lj_out))
            if self.bonded is not None:
                self._bonded_forces()
            self.L.kor_limit(self.n, _p(self.eps), _p(self.sig), self.limit, _p(self.f))
            if self.use_atm:
                self.atm_forces(with_atm_virial)
            return
        pairs, shifts = self.pair_list()
        self.ncount = np.zeros(self.n, np.int64) if ncount else None
        if self.use_lj:
            self.hist = None
            if nbins > 0:
                self.hist = (np.zeros(nbins), np.zeros(nbins), np.zeros(nbins, np.uint64), np.zeros(nbins, np.uint64))
            h = self.hist
            self.L.kor_lj(C.byref(self.g), pairs.shape[0], _p(pairs), _p(shifts), _p(self.r), _p(self.eps),
                          _p(self.sig), _p(self.id), self.cutoff, self.virial_mode, _p(self.f),
                          _p(self.ncount) if ncount else None, C.byref(self.lj_out), nbins, max_sigma,
                          _p(h[0]) if h else None, _p(h[1]) if h else None, _p(h[2]) if h else None,
                          _p(h[3]) if h else None)
        if self.table is not None:
            tx, ty, lo, hi = self.table
            self.L.kor_pair_table(pairs.shape[0], _p(pairs), _p(shifts), _p(self.r), self.cutoff, tx.size, _p(tx),
                                  _p(ty), lo, hi, _p(self.f))
        if self.use_fene:
            self.L.kor_fene(pairs.shape[0], _p(pairs), _p(shifts), _p(self.r), _p(self.eps), _p(self.sig),
                            _p(self.id), self.stiffness, _p(self.f))
        if self.bonded is not None:
            self._bonded_forces()
        self.L.kor_limit(self.n, _p(self.eps), _p(self.sig), self.limit, _p(self.f))
        if self.use_atm:
            self.atm_forces(with_atm_virial)

    def _bonded_forces(self):
        b = self.bonded
        bonds = np.ascontiguousarray(b["bonds"], np.int64)
        angles = np.ascontiguousarray(b["angles"], np.int64)
        w = np.zeros(6)
        self.e_bonded = self.L.kor_bonded(bonds.shape[0], _p(bonds), b["kb"], b["r0"], angles.shape[0],
                                          _p(angles), b["ka"], b["theta0"], _p(self.r), None, _p(self.f), _p(w))
        self.w_bonded = w

    def atm_forces(self, with_virial=False):
        if self.atm_mode == "compat":
            self.L.kor_atm_compat(C.byref(self.g), C.byref(self.cells), _p(self.r), self.nu, self.cutoff_atm,
                                  self.atm_sign, self.virial_mode, int(with_virial), _p(self.f), C.byref(self.atm_out))
        else:
            self.L.kor_atm_vertex(C.byref(self.g), C.byref(self.cells), _p(self.r), self.nu, self.cutoff_atm,
                                  self.atm_sign, 1 if self.atm_mode == "vertex_compat" else 0, _p(self.f),
                                  C.byref(self.atm_out))

    # --- integration & sensors ---------------------------------------------
    def integrate0(self):
        self.L.kor_step0(self.n, _p(self.r), _p(self.v), _p(self.f), _p(self.m), self.dt)

    def integrate1(self):
        self.L.kor_step1(self.n, _p(self.v), _p(self.f), _p(self.m), self.dt)

    def step(self, first=False, listless=False):
        if not first:
            self.integrate0()
        self.update_container()
        self.forces(listless=listless)
        if not first:
            self.integrate1()

    def temperature(self):
        return self.L.kor_temperature(self.n, _p(self.r), _p(self.v), _p(self.m), _p(self.low), _p(self.high))

    def momentum(self, n_terms=None):
        acc = np.zeros(6)
        self.L.kor_momentum(self.n_mol if n_terms is None else n_terms, _p(self.v), _p(self.m), _p(acc))
        return acc

    def rdf_profile(self, max_r, nbins):
        """RDF_Profiler::measure + getRDF for one sample (plugins/IBI/RDF_Profiler.cpp:18-55):
        raw histogram with dr = max_r / nbins, then the normalised g(r)."""
        bins = np.zeros(nbins)
        com = np.zeros((self.n_mol, 3))
        self.L.kor_com(self.n_mol, _p(self.mol_off), _p(self.r), _p(self.m), _p(com))
        box = (self.high - self.low).copy()
        dr = max_r / nbins
        self.L.kor_rdf(self.n_mol, _p(com), _p(box), max_r, dr, nbins, _p(bins))
        return bins, rdf_profile_normalise(bins, 1, max_r, nbins, self.n_mol, float(np.prod(box)))

    def rdf(self, max_r, dr):
        nb = int(self.L.kor_rdf_nbins(max_r, dr))
        bins = np.zeros(nb)
        com = np.zeros((self.n_mol, 3))
        self.L.kor_com(self.n_mol, _p(self.mol_off), _p(self.r), _p(self.m), _p(com))
        box = (self.high - self.low).copy()
        self.L.kor_rdf(self.n_mol, _p(com), _p(box), max_r, dr, nb, _p(bins))
        return bins


def comp_force(nu, a, b, c):
    return lib().kor_atm_comp_force(nu, a, b, c)


def atm_energy(nu, a, b, c):
    return lib().kor_atm_energy(nu, a, b, c)


def pressure_factor():
    return lib().kor_pressure_factor()


# --- three-body surrogate (no reference counterpart) ------------------------
SUR_NF, SUR_H = 32, 64
SUR_NPARAM = SUR_H * SUR_NF + SUR_H + SUR_H * SUR_H + SUR_H + SUR_H + 1


def _sur_lib():
    L = lib()
    if not getattr(L, "_sur", False):
        L.kor_sur_features.argtypes = [C.c_int, P, D, P]
        L.kor_sur_mlp.argtypes = [P, P, P]
        L.kor_sur_mlp.restype = D
        L.kor_sur_mlp_param_grad.argtypes = [P, P, P]
        L.kor_sur_energy_forces.argtypes = [I64, P, P, D, P, P, P, D, D, P, P]
        L.kor_sur_energy_forces.restype = D
        L._sur = True
    return L


def sur_features(d, rc=2.0):
    d = np.ascontiguousarray(d, np.float64).reshape(-1, 3)
    raw = np.zeros(SUR_NF)
    _sur_lib().kor_sur_features(d.shape[0], _p(d), rc, _p(raw))
    return raw


def sur_mlp(params, x):
    params = np.ascontiguousarray(params, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    dx = np.zeros(SUR_NF)
    e = _sur_lib().kor_sur_mlp(_p(params), _p(x), _p(dx))
    return e, dx


def sur_mlp_param_grad(params, x):
    params = np.ascontiguousarray(params, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    g = np.zeros(SUR_NPARAM)
    _sur_lib().kor_sur_mlp_param_grad(_p(params), _p(x), _p(g))
    return g


def sur_energy_forces(r, box, params, fmean, fstd, e_scale, e_shift, rc=2.0):
    r = np.ascontiguousarray(r, np.float64)
    n = r.shape[0]
    box = np.ascontiguousarray(box, np.float64)
    e = np.zeros(n)
    f = np.zeros((n, 3))
    et = _sur_lib().kor_sur_energy_forces(n, _p(r), _p(box), rc, _p(np.ascontiguousarray(params, np.float64)),
                                          _p(np.ascontiguousarray(fmean, np.float64)),
                                          _p(np.ascontiguousarray(fstd, np.float64)), e_scale, e_shift, _p(e), _p(f))
    return et, e, f


def atm2b_factor(nu, n_mol, volume, eps, sig):
    """ATM2B::ATM2B's potential_factor (kor_atm2b_factor)."""
    return lib().kor_atm2b_factor(float(nu), float(n_mol), float(volume), float(eps), float(sig))


def rdf_profile_normalise(bins, samples, max_r, nbins, n, volume):
    """RDF_Profiler::getRDF (RDF_Profiler.cpp:34-52): bins / samples / (N (N-1) V_bin / V)."""
    dr = max_r / nbins
    out = np.zeros(nbins)
    for b in range(nbins):
        rmin, rmax = b * dr, (b + 1) * dr
        binvol = (4.0 / 3.0) * np.pi * (rmax * rmax * rmax - rmin * rmin * rmin)
        den = n * (n - 1.0) * binvol / volume
        out[b] = bins[b] / samples / den
    return out


def visc_green_kubo(series, dt, origin_free):
    """ViscositySensor::TensorEvaluator::integrate (sensors/ViscositySensor.cpp:118-159)
    for the bulk (XX YY ZZ) and shear (XY XZ YZ) components of a series of
    pressure tensors / V (rows in the order XX XY YY XZ YZ ZZ): per component
    c(k) = mean_t (p(t) - s)(p(t+k) - s) (s = mean p when origin_free), the
    integral (c(0) + c(n-1) + sum of the inner c(k)) dt / 2, averaged."""
    p_all = np.asarray(series, np.float64)
    out = []
    for dims in ((0, 2, 5), (1, 3, 4)):
        acc = 0.0
        for d in dims:
            p = p_all[:, d]
            n = p.size
            s = p.mean() if origin_free else 0.0
            q = p - s
            c = np.array([np.dot(q[:n - k], q[k:]) / (n - k) for k in range(n)])
            acc += (c[0] + c[-1] + c[1:-1].sum()) * dt / 2.0
        out.append(acc / len(dims))
    return tuple(out)


def visc_factor(volume, temperature):
    """ViscositySensor::write's unit factor (Da_kg^2 A_m / ps_s^3) * V / (kB T)."""
    return (1.66053906892e-27 ** 2 * 1e-10 / 1e-36) * volume / (1.380649e-23 * temperature)


# --- IBI plugin (plugins/IBI/*.cpp) under the stock main's loop ---------------

def ibi_continue_below(y, k0):
    """Linear continuation below node k0 with the slope of (k0, k0 + 1)
    (IBI.cpp:140-150 and 170-180)."""
    if k0 < 0:
        return
    dy = y[k0 + 1] - y[k0] if k0 + 1 < y.size else 0.0
    v = y[k0]
    for k in range(k0, -1, -1):
        y[k] = v
        v -= dy


def ibi_initial_potential(g0, temperature):
    """IBI::initializePotentialValues (IBI.cpp:130-153): U0 = -T ln g0, continued
    linearly below the first finite value."""
    with np.errstate(divide="ignore", invalid="ignore"):
        u = -temperature * np.log(np.asarray(g0, np.float64))
    fin = np.flatnonzero(np.isfinite(u))
    ibi_continue_below(u, int(fin[0]) if fin.size else -1)
    return u


def ibi_correction(pot, g_i, g0, alpha, temperature):
    """IBI::addPotentialCorrection (IBI.cpp:155-182): (new potential, update)."""
    pot = np.asarray(pot, np.float64).copy()
    with np.errstate(divide="ignore", invalid="ignore"):
        d = alpha * temperature * np.log(np.asarray(g_i) / np.asarray(g0))
    ok = np.isfinite(d)
    pot[ok] += d[ok]
    update = np.where(ok, d, 0.0)
    nz = np.flatnonzero(np.asarray(g0) != 0.0)
    ibi_continue_below(pot, int(nz[0]) if nz.size else -1)
    return pot, update


def ibi_force(x, pot):
    """IBI::derivativeOfPotential (IBI.cpp:184-191) with FunctionPL::derivative
    (IBI_Math.cpp:21-33): F = -dU/dr, one-sided at the ends, central inside."""
    x, y = np.asarray(x, np.float64), np.asarray(pot, np.float64)
    d = np.empty_like(y)
    d[0] = (y[1] - y[0]) / (x[1] - x[0])
    d[-1] = (y[-1] - y[-2]) / (x[-1] - x[-2])
    d[1:-1] = (y[2:] - y[:-2]) / (x[2:] - x[:-2])
    return -d


def ibi_convergence(mode, x, g0, g_i):
    """IBI::Convergence::integral / l2 (IBI.cpp:210-253)."""
    g0, g_i = np.asarray(g0, np.float64), np.asarray(g_i, np.float64)
    if mode == "l2":
        return float(np.sum((g0 - g_i) ** 2))
    dx = np.diff(np.asarray(x, np.float64))
    a, b = np.abs(g_i - g0), np.abs(g_i + g0)
    diff = float(np.sum(dx * (a[1:] + a[:-1]) / 2.0))
    tot = float(np.sum(dx * (b[1:] + b[:-1]) / 2.0))
    return 1.0 - diff / (tot if tot != 0 else 1e-15)


def ibi_should_stop(values, mode, stop, threshold, window):
    """IBI::Convergence::shouldStop (IBI.cpp:262-281)."""
    n = len(values)
    if stop == "worse":
        if n < 2:
            return False
        prev, last = values[-2], values[-1]
        if mode == "l2":
            return not (prev > threshold) and not (prev >= last)
        return not (prev < threshold) and not (prev <= last)
    if n < window:
        return False
    tail = values[n - window:]
    return all((v <= threshold) if mode == "l2" else (v >= threshold) for v in tail)


def run_ibi(sim, temperature, steps, bins, alpha, steps_equil, steps_measure, conv_mode="integral",
            conv_stop="worse", conv_threshold=0.99, conv_window=10):
    """The stock main's Simulation::run (Simulation.cpp:10-80) with the
    VelocityScaling thermostat and the IBI plugin's post_forces state machine
    (IBI.cpp:28-118) on an OracleSim (LJ until the first RDF is complete, then
    the tabulated force alone).  Returns the files IBI writes ({name: (x, y)}),
    the convergence values, whether the plugin stopped the run and the final
    step count."""
    max_r = sim.cutoff
    nodes = (np.arange(bins) + 0.5) * (max_r / bins)
    volume = float(np.prod(sim.high - sim.low))
    st = dict(phase="init", cur=0, it=0, acc=np.zeros(bins), samples=0.0, g0=None, pot=None, conv=[],
              max_step=steps, stop=False)
    files = {}

    def rdf():
        return rdf_profile_normalise(st["acc"], st["samples"], max_r, bins, sim.n_mol, volume)

    def measure():
        b, _ = sim.rdf_profile(max_r, bins)
        st["acc"] += b
        st["samples"] += 1.0

    def set_force():
        f = ibi_force(nodes, st["pot"])
        files[f"force_{st['it']}"] = (nodes, f)
        # IBI.cpp:50-54: the tabulated force replaces every functor (LJ, FENE, Limit)
        sim.use_lj = sim.use_fene = sim.use_atm = False
        sim.limit = np.inf
        sim.table = (nodes.copy(), f, 1e6, 0.0)

    def post_forces(simstep):
        st["cur"] += 1
        if st["phase"] == "init":
            if st["cur"] < steps_measure:
                measure()
                return
            st.update(phase="equil", cur=0, it=0)
            st["g0"] = rdf()
            files["rdf_0"] = (nodes, st["g0"])
            st["acc"][:] = 0.0
            st["samples"] = 0.0
            st["pot"] = ibi_initial_potential(st["g0"], temperature)
            files["pot_0"] = (nodes, st["pot"].copy())
            set_force()
        elif st["phase"] == "equil":
            if st["cur"] < steps_equil:
                return
            st.update(phase="measure", cur=0)
        else:
            if st["cur"] < steps_measure:
                measure()
                return
            st.update(phase="equil", cur=0)
            g_i = rdf()
            st["pot"], upd = ibi_correction(st["pot"], g_i, st["g0"], alpha, temperature)
            files[f"update_{st['it']}"] = (nodes, upd)
            st["it"] += 1
            files[f"pot_{st['it']}"] = (nodes, st["pot"].copy())
            set_force()
            files[f"rdf_{st['it']}"] = (nodes, g_i)
            st["conv"].append(ibi_convergence(conv_mode, nodes, st["g0"], g_i))
            if ibi_should_stop(st["conv"], conv_mode, conv_stop, conv_threshold, conv_window):
                st["max_step"] = simstep
                st["stop"] = True
                return
            st["acc"][:] = 0.0
            st["samples"] = 0.0

    sim.update_container()
    sim.forces()
    post_forces(0)
    sim.thermostat(temperature)
    simstep = 0
    while simstep < st["max_step"]:
        sim.integrate0()
        sim.update_container()
        sim.forces()
        post_forces(simstep)
        sim.integrate1()
        simstep += 1
        sim.thermostat(temperature)
    if st["pot"] is not None:
        files["final_pot"] = (nodes, st["pot"].copy())
    return files, st["conv"], st["stop"], simstep

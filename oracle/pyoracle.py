"""Python access to the ORACLE (test infrastructure, never the product).

Two implementations with one interface:

* :class:`Oracle` -- the C restatement in ``oracle/mhd_oracle.c`` (run-time
  grid sizes; builds on x86 and Arm; OpenMP threads).
* :class:`RefOracle` -- the reference's own C sources compiled in place into
  ``oracle/_ref/`` by ``oracle/build_ref.py`` (one library per grid size; only
  where the reference tree exists).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use this
module, as the checker or the CPU baseline.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmhd_oracle.so")

GRIDSPEC_FIELDS = ["ix", "jy", "kz", "x0", "dx0", "lx", "y0", "ly", "z0", "dz0", "lz",
                   "stretchratio", "dxmax", "dzmax", "rin"]
PARAM_FIELDS = ["cfl", "dtmin", "rhocr", "prcr", "betacr", "epssp0", "tausp", "scalez",
                "scaler", "scalephase", "armnum", "omegasp", "omegapattern", "pitch"]
FLAG_FIELDS = ["limiter", "solver", "scheme", "cooling", "gravity", "source"]


class _GridSpec(C.Structure):
    _fields_ = [("nr", C.c_int), ("nphi", C.c_int), ("nz", C.c_int)] + \
               [(f, C.c_double) for f in GRIDSPEC_FIELDS[3:]]


class _Params(C.Structure):
    _fields_ = [(f, C.c_double) for f in PARAM_FIELDS] + [(f, C.c_int) for f in FLAG_FIELDS]


# ---------------------------------------------------------------------------
# the benchmark's disc workloads, defined here too so that the CPU legs (the
# reference arm and the CPU baseline) run without loading the product library
# ---------------------------------------------------------------------------

def default_params(**over):
    """The reference's knobs (input.h:58-102, constant.h:62-79) as a dict."""
    year, t0, kpc = 3.1536e+7, 4.7058e+15, 3.08568e+21
    omega0, oneokpc = 1.0 / t0, 1.0 / kpc
    p = dict(cfl=0.4, dtmin=1.0e-9, rhocr=1.0e-4, prcr=0.015, betacr=0.1, epssp0=0.05,
             tausp=200.0 * 1.0e+6 * year / t0, scalez=0.03, scaler=0.7, scalephase=0.1, armnum=2.0,
             omegasp=10.0e+5 / omega0 * oneokpc, omegapattern=10.0e+5 / omega0 * oneokpc,
             pitch=15.0 * np.pi / 180.0, limiter=0, solver=0, scheme=2, cooling=1, gravity=1, source=0)
    named = {"limiter": {"minmod": 0, "mc": 1, "vanleer": 2, "superbee": 3},
             "solver": {"hlld": 0, "hll": 1}}
    for k, v in over.items():
        if k in named and isinstance(v, str):
            v = named[k][v]
        if k == "precision":
            continue
        p[k] = float(v) if k == "armnum" else v
    return p


def gridspec_disc(nr, nphi, nz):
    """The uniform disc grid r in [0.1,1.5], phi in [0,2pi), z in [-0.5,0.5]
    in the reference's input.h terms (x0 = first cell centre, stretching
    pushed beyond the domain)."""
    dx0, dz0 = 1.4 / nr, 1.0 / nz
    return dict(ix=nr, jy=nphi, kz=nz, x0=0.1 + 0.5 * dx0, dx0=dx0, lx=1.0e30, y0=0.0, ly=2.0 * np.pi,
                z0=-0.5 + 0.5 * dz0, dz0=dz0, lz=1.0e30, stretchratio=1.05, dxmax=50.0 * dx0,
                dzmax=50.0 * dz0, rin=0.1)


def workload(name, nr=None, nphi=None, nz=None, **over):
    """dims, params dict and initial-condition arguments of a named disc
    workload (the same definitions as the product binding's workload())."""
    base = dict(limiter="minmod", solver="hlld", scheme=3, cooling=0, gravity=0, prcr=1.0e-3,
                rhocr=1.0e-4, betacr=0.1, cfl=0.4, omegasp=0.0)
    if name == "disc1":
        dims, beta = (64, 64, 32), 10.0
    elif name == "disc2":
        dims, beta = (256, 256, 128), 1.0
        base.update(limiter="mc", gravity=1, cooling=1, epssp0=0.03, omegapattern=0.5,
                    pitch=15.0 * np.pi / 180.0, armnum=2)
    elif name == "disc3":
        dims, beta = (256, 256, 128), 10.0
    elif name == "disc5":
        dims, beta = (512, 512, 256), 1.0
        base.update(cooling=1)
    else:
        raise ValueError(name)
    dims = (nr or dims[0], nphi or dims[1], nz or dims[2])
    beta = over.pop("beta", beta)
    base.update(over)
    return dims, default_params(**base), dict(beta=beta, amp=0.01, seed=0)


def build_oracle(force=False):
    """Compile oracle/mhd_oracle.c (here or on the GPU machine) and return the path."""
    src = os.path.join(HERE, "mhd_oracle.c")
    hdr = os.path.join(HERE, "mhd_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-fPIC", "-shared", src, "-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _Common:
    """Shared array-shape bookkeeping."""

    def _shapes(self, dims):
        self.ix, self.jy, self.kz, self.ixmax, self.jymax, self.kzmax, self.irin = [int(v) for v in dims]
        self.cell = (self.ixmax, self.jymax, self.kzmax)
        self.face = (self.ixmax - 1, self.jymax - 1, self.kzmax - 1)
        self.nc = self.ixmax * self.jymax * self.kzmax

    def grid1d(self):
        a = [np.zeros(self.ixmax) for _ in range(7)]
        y = np.zeros(self.jymax)
        zz = [np.zeros(self.kzmax) for _ in range(5)]
        sc = np.zeros(4)
        self._get_grid1d(*a, y, *zz, sc)
        names = ["x", "xm", "dx", "dxm", "oneox", "oneoxm", "oneodx"]
        out = dict(zip(names, a))
        out["oneoxm"] = out["oneoxm"][:-1]
        out["y"] = y
        out.update(zip(["z", "zm", "dz", "dzm", "oneodz"], zz))
        out.update(dict(zip(["dy", "oneody", "minminlength", "oneominminlength"], sc)))
        return out

    def metric(self):
        g = np.zeros((6,) + self.face)
        ml = np.zeros(self.cell)
        xa = np.zeros(11)
        za = np.zeros(11)
        ca = np.zeros((self.irin + 1, self.kzmax))
        kr = np.zeros(self.irin + 1, dtype=np.int32)
        self._get_metric(g, ml, xa, za, ca, kr)
        return dict(g=g, minlength=ml, xabs=xa, zabs=za, cabs=ca, krin=kr)

    def load(self, U, V, Uinit=None, Vinit=None, rhofloor=None, rhocr=None):
        U = _f64(U)
        V = _f64(V)
        Uinit = U if Uinit is None else _f64(Uinit)
        Vinit = V if Vinit is None else _f64(Vinit)
        if rhofloor is None:
            rhofloor = U[0] * (self.rhocr if rhocr is None else rhocr)
        self._load(U, V, Uinit, Vinit, _f64(rhofloor))

    def store(self):
        U = np.zeros((9,) + self.cell)
        V = np.zeros((9,) + self.cell)
        U1 = np.zeros((9,) + self.cell)
        self._store(U, V, U1)
        return U, V, U1

    def limiter(self, d):
        Vl = np.zeros((9,) + self.face)
        Vr = np.zeros((9,) + self.face)
        self._limiter(d, Vl, Vr)
        return Vl, Vr

    def flux(self, d):
        F = np.zeros((9,) + self.face)
        self._flux(d, F)
        return F

    def source(self):
        S = np.zeros((9,) + self.cell)
        self._source(S)
        return S

    def gravity(self):
        axi = np.zeros((3,) + self.cell)
        gr = np.zeros((3,) + self.cell)
        self._get_gravity(axi, gr)
        return axi, gr

    def utov_check(self, U):
        U = _f64(U).copy()
        V = np.zeros((9,) + self.cell)
        cnt = np.zeros(3, dtype=np.int32)
        self._utov_check(U, V, cnt)
        return U, V, cnt


class Oracle(_Common):
    """The C restatement (oracle/mhd_oracle.c)."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(build_oracle())
            vp = C.c_void_p
            lib.orc_create.restype = vp
            lib.orc_create.argtypes = [C.POINTER(_GridSpec), C.POINTER(_Params)]
            lib.orc_destroy.argtypes = [vp]
            lib.orc_dims.argtypes = [vp, _IP]
            lib.orc_set_threads.argtypes = [C.c_int]
            lib.orc_get_grid1d.argtypes = [vp] + [_DP] * 14
            lib.orc_get_metric.argtypes = [vp, _DP, _DP, _DP, _DP, _DP, _IP]
            lib.orc_initial_gravity.argtypes = [vp]
            lib.orc_set_gravity_axi.argtypes = [vp, _DP]
            lib.orc_get_gravity.argtypes = [vp, _DP, _DP]
            lib.orc_load.argtypes = [vp, _DP, _DP, _DP, _DP, _DP]
            lib.orc_store.argtypes = [vp, _DP, _DP, _DP]
            lib.orc_setdt.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), _IP]
            lib.orc_spiral_gravity.argtypes = [vp, C.c_double]
            lib.orc_step.restype = C.c_int
            lib.orc_step.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), _IP]
            lib.orc_set_dtch.argtypes = [vp, C.c_double, C.c_double, C.c_double]
            lib.orc_limiter.argtypes = [vp, C.c_int, _DP, _DP]
            lib.orc_flux.argtypes = [vp, C.c_int, _DP]
            lib.orc_source.argtypes = [vp, _DP]
            lib.orc_utov_check.argtypes = [vp, _DP, _DP, _IP]
            lib.orc_cooling.restype = C.c_int
            lib.orc_cooling.argtypes = [C.c_double, C.c_double]
            lib.orc_ic_disc.argtypes = [vp, C.c_double, C.c_double, C.c_ulonglong]
            cls._lib = lib
        return cls._lib

    def __init__(self, gridspec, params, threads=None):
        lib = self.lib()
        self.threads = int(threads or os.cpu_count() or 1)
        gs = _GridSpec(*[gridspec[f] for f in GRIDSPEC_FIELDS])
        pr = _Params(*([float(params[f]) for f in PARAM_FIELDS] + [int(params[f]) for f in FLAG_FIELDS]))
        self.rhocr = float(params["rhocr"])
        self.h = lib.orc_create(C.byref(gs), C.byref(pr))
        if not self.h:
            raise MemoryError("orc_create failed")
        dims = np.zeros(7, dtype=np.int32)
        lib.orc_dims(self.h, dims)
        self._shapes(dims)
        h = self.h
        self._get_grid1d = lambda *a: lib.orc_get_grid1d(h, *a)
        self._get_metric = lambda *a: lib.orc_get_metric(h, *a)
        self._load = lambda *a: lib.orc_load(h, *a)
        self._store = lambda *a: lib.orc_store(h, *a)
        self._limiter = lambda d, *a: lib.orc_limiter(h, d, *a)
        self._flux = lambda d, *a: lib.orc_flux(h, d, *a)
        self._source = lambda *a: lib.orc_source(h, *a)
        self._get_gravity = lambda *a: lib.orc_get_gravity(h, *a)
        self._utov_check = lambda *a: lib.orc_utov_check(h, *a)

    def close(self):
        if getattr(self, "h", None):
            self.lib().orc_destroy(self.h)
            self.h = None

    __del__ = close

    def initial_gravity(self):
        self.lib().orc_initial_gravity(self.h)

    def ic_disc(self, beta, amp=0.01, seed=0):
        """The seeded disc state set in place (orc_ic_disc): V, U, the
        initial copies and the density floor."""
        self.lib().orc_set_threads(self.threads)
        self.lib().orc_ic_disc(self.h, float(beta), float(amp), int(seed))

    def set_gravity_axi(self, axi):
        self.lib().orc_set_gravity_axi(self.h, _f64(axi))

    def setdt(self):
        dt, ch = C.c_double(), C.c_double()
        ijk = np.zeros(3, dtype=np.int32)
        self.lib().orc_setdt(self.h, C.byref(dt), C.byref(ch), ijk)
        return dt.value, ch.value, tuple(int(v) for v in ijk)

    def spiral(self, t):
        self.lib().orc_spiral_gravity(self.h, float(t))

    def set_dtch(self, dt, ch, psicoef=1.0):
        self.lib().orc_set_dtch(self.h, dt, ch, psicoef)

    def step(self, t):
        # the OpenMP thread count is process-wide state shared with RefOracle
        self.lib().orc_set_threads(self.threads)
        tt, dt, ch = C.c_double(t), C.c_double(), C.c_double()
        cnt = np.zeros(3, dtype=np.int32)
        rc = self.lib().orc_step(self.h, C.byref(tt), C.byref(dt), C.byref(ch), cnt)
        return rc, tt.value, dt.value, ch.value, cnt


class RefOracle(_Common):
    """The reference's own C, compiled in place (oracle/_ref/, this container only)."""

    def __init__(self, nr, nphi, nz, params, shipped=False):
        import build_ref  # noqa: local module in oracle/
        path = build_ref.build(nr, nphi, nz, shipped=shipped)
        lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        vp = None
        lib.ref_dims.argtypes = [_IP]
        lib.ref_set_params.argtypes = [_DP, _IP]
        lib.ref_get_grid1d.argtypes = [_DP] * 14
        lib.ref_get_metric.argtypes = [_DP, _DP, _DP, _DP, _DP, _IP]
        lib.ref_get_gravity.argtypes = [_DP, _DP]
        lib.ref_set_gravity_axi.argtypes = [_DP]
        lib.ref_load.argtypes = [_DP] * 5
        lib.ref_store.argtypes = [_DP, _DP, _DP]
        lib.ref_setdt.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.ref_spiral_gravity.argtypes = [C.c_double]
        lib.ref_step.restype = C.c_int
        lib.ref_step.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), _IP]
        lib.ref_set_dtch.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.ref_limiter.argtypes = [C.c_int, _DP, _DP]
        lib.ref_flux.argtypes = [C.c_int, _DP]
        lib.ref_source.argtypes = [_DP]
        lib.ref_utov_check.argtypes = [_DP, _DP, _IP]
        lib.ref_cooling.restype = C.c_int
        lib.ref_cooling.argtypes = [C.c_double, C.c_double]
        lib.ref_get_initial.argtypes = [_DP, _DP, _DP]
        lib.ref_set_threads.argtypes = [C.c_int]
        lib.ref_set_threads(1)
        lib.ref_binary_output.argtypes = [C.c_int, C.c_double]
        lib.ref_restart_read.argtypes = [C.c_int]
        lib.ref_text_output.argtypes = [C.c_int, C.c_int, C.c_double]
        lib.ref_check_flags.argtypes = [_IP]
        self.lib = lib
        self.rhocr = float(params["rhocr"])
        p = np.array([float(params[f]) for f in PARAM_FIELDS])
        fl = np.array([int(params[f]) for f in FLAG_FIELDS], dtype=np.int32)
        lib.ref_reset()
        lib.ref_set_params(p, fl)
        lib.ref_grid()
        dims = np.zeros(7, dtype=np.int32)
        lib.ref_dims(dims)
        self._shapes(dims)
        self._get_grid1d = lib.ref_get_grid1d
        self._get_metric = lib.ref_get_metric
        self._load = lib.ref_load
        self._store = lib.ref_store
        self._limiter = lib.ref_limiter
        self._flux = lib.ref_flux
        self._source = lib.ref_source
        self._get_gravity = lib.ref_get_gravity
        self._utov_check = lib.ref_utov_check
        del vp

    def close(self):
        pass

    def binary_output(self, num, t):
        """BinaryOutput() into ./<num>/ of the current working directory."""
        self.lib.ref_binary_output(int(num), float(t))

    def text_output(self, num, nstep, t):
        """GNUOutputCylinder() + GDLOutputCylinder() into the working directory."""
        self.lib.ref_text_output(int(num), int(nstep), float(t))

    def restart_read(self, num):
        """RestartRead(num) from ./<num>/: V from the files, VtoU, Check;
        returns Check's floor counters."""
        self.lib.ref_set_threads(1)
        self.lib.ref_restart_read(int(num))
        cnt = np.zeros(3, dtype=np.int32)
        self.lib.ref_check_flags(cnt)
        return cnt

    def save_initial(self):
        self.lib.ref_save_initial()

    def galactic_disc3(self):
        """GalacticDisc3() (model.h:149-327): sets V, U, the initial arrays and
        the axisymmetric gravity in the reference's globals."""
        self.lib.ref_galactic_disc3()

    def get_initial(self):
        shp = (9,) + self.cell
        Ui, Vi, rf = np.zeros(shp), np.zeros(shp), np.zeros(self.cell)
        self.lib.ref_get_initial(Ui, Vi, rf)
        return Ui, Vi, rf

    def initial_gravity(self):
        self.lib.ref_initial_gravity()

    def set_gravity_axi(self, axi):
        self.lib.ref_set_gravity_axi(_f64(axi))

    def setdt(self):
        dt, ch = C.c_double(), C.c_double()
        self.lib.ref_setdt(C.byref(dt), C.byref(ch))
        return dt.value, ch.value, None

    def spiral(self, t):
        self.lib.ref_spiral_gravity(float(t))

    def set_dtch(self, dt, ch, psicoef=1.0):
        self.lib.ref_set_dtch(dt, ch, psicoef)

    def step(self, t):
        # Setdt and Check share running max / counters between OpenMP threads
        # without synchronisation (setdt.h:60-69, check.h:53,96,139): one thread
        self.lib.ref_set_threads(1)
        tt, dt, ch = C.c_double(t), C.c_double(), C.c_double()
        cnt = np.zeros(3, dtype=np.int32)
        rc = self.lib.ref_step(C.byref(tt), C.byref(dt), C.byref(ch), cnt)
        return rc, tt.value, dt.value, ch.value, cnt

"""ctypes binding of libmhdgpu.so (include/mhd_gpu.h) plus the synthetic disc
workloads used by the tests and the benchmark.

The library is the product: CUDA kernels for sm_103a behind a C-ABI, with the
host set-up helpers of the reference (grid, gravity, initial condition).  This
module only marshals arrays; every step runs in the library.  If the library
is missing it raises -- there is no Python or CPU fallback.
"""
import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(PKG, "lib", "libmhdgpu.so")

MHD_OK = 0
MHD_ERR_ARG = -1
MHD_ERR_DT = -3
MHD_ERR_TIMEOUT = -6
MHD_ERR_IO = -8
LIMITER = {"minmod": 0, "mc": 1, "vanleer": 2, "superbee": 3}
SOURCE = {"spiral": 0, "axi": 1, "uniformgz": 2, "none": 3}
SOLVER = {"hlld": 0, "hll": 1}
PREC = {"fp64": 0, "fp32": 1, "fp32x2": 2}


class MhdParams(C.Structure):
    _fields_ = [("cfl", C.c_double), ("dtmin", C.c_double), ("rhocr", C.c_double),
                ("prcr", C.c_double), ("betacr", C.c_double), ("epssp0", C.c_double),
                ("tausp", C.c_double), ("scalez", C.c_double), ("scaler", C.c_double),
                ("scalephase", C.c_double), ("armnum", C.c_int), ("omegasp", C.c_double),
                ("omegapattern", C.c_double), ("pitch", C.c_double), ("limiter", C.c_int),
                ("solver", C.c_int), ("scheme", C.c_int), ("cooling", C.c_int),
                ("gravity", C.c_int), ("precision", C.c_int), ("source", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class MhdGridSpec(C.Structure):
    _fields_ = [("ix", C.c_int), ("jy", C.c_int), ("kz", C.c_int)] + [
        (f, C.c_double) for f in ["x0", "dx0", "lx", "y0", "ly", "z0", "dz0", "lz",
                                  "stretchratio", "dxmax", "dzmax", "rin"]]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_PD = C.POINTER(C.c_double)


class MhdGrid(C.Structure):
    _fields_ = [("ix", C.c_int), ("jy", C.c_int), ("kz", C.c_int), ("irin", C.c_int),
                ("compact", C.c_int), ("dx0", C.c_double), ("rin", C.c_double),
                ("x", _PD), ("xm", _PD), ("dx", _PD), ("dxm", _PD), ("oneox", _PD),
                ("oneodx", _PD), ("y", _PD), ("dy", C.c_double), ("oneody", C.c_double),
                ("z", _PD), ("zm", _PD), ("dz", _PD), ("dzm", _PD), ("oneodz", _PD),
                ("g1", _PD), ("g2", _PD), ("g3", _PD), ("g4", _PD), ("g5", _PD), ("g6", _PD),
                ("minlength", _PD), ("minminlength", C.c_double),
                ("x_absorb_factor", _PD), ("z_absorb_factor", _PD), ("c_absorb_factor", _PD),
                ("Grxaxi", _PD), ("Gryaxi", _PD), ("Grzaxi", _PD)]


class MhdDiag(C.Structure):
    _fields_ = [("mass", C.c_double), ("angmom", C.c_double), ("energy", C.c_double),
                ("psi", C.c_double), ("maxdivb", C.c_double)]


_lib = None


def lib():
    """Load libmhdgpu.so (built by build.py).  Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError("libmhdgpu.so is not built (%s); run __graft_entry__.build()" % LIBPATH)
    L = C.CDLL(LIBPATH)
    vp = C.c_void_p
    DP = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
    IP = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    sig = {
        "mhd_errstr": (C.c_char_p, [C.c_int]),
        "mhd_params_default": (None, [C.POINTER(MhdParams)]),
        "mhd_gridspec_disc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(MhdGridSpec)]),
        "mhd_gridspec_shipped": (C.c_int, [C.POINTER(MhdGridSpec)]),
        "mhd_grid_storage": (C.c_size_t, [C.POINTER(MhdGridSpec)]),
        "mhd_grid_build": (C.c_int, [C.POINTER(MhdGridSpec), DP, C.POINTER(MhdGrid)]),
        "mhd_initial_gravity": (C.c_int, [C.POINTER(MhdGrid), DP, DP, DP]),
        "mhd_ic_disc": (C.c_int, [C.POINTER(MhdGrid), C.c_double, C.c_double, C.c_ulonglong,
                                  C.c_double, vp, vp, vp, vp, vp]),
        "mhd_vtou": (C.c_int, [C.POINTER(MhdGrid), DP, DP]),
        "mhd_ic_galactic_disc3": (C.c_int, [C.POINTER(MhdGrid), C.POINTER(MhdParams), vp, vp, vp, vp, vp]),
        "mhd_binary_output": (C.c_int, [C.c_char_p, C.c_int, C.c_double, C.POINTER(MhdGrid), DP]),
        "mhd_binary_output_arrays": (C.c_int, [C.c_char_p, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                               DP, DP, DP, DP]),
        "mhd_restart_read": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, DP]),
        "mhd_check": (C.c_int, [C.POINTER(MhdGrid), C.POINTER(MhdParams), DP, DP, DP, vp]),
        "mhd_save_initial": (C.c_int, [C.POINTER(MhdGrid), C.c_double, DP, DP, vp, vp, vp]),
        "mhd_restart": (C.c_int, [C.c_char_p, C.c_int, C.c_double, C.POINTER(MhdGrid), C.POINTER(MhdParams),
                                  DP, DP, DP, DP, DP, _PD, _PD]),
        "mhd_gnu_output_cylinder": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_double, C.POINTER(MhdGrid),
                                              DP, DP]),
        "mhd_gdl_output_cylinder": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(MhdGrid), DP]),
        "mhd_checkpoint_begin": (C.c_int, [vp, C.c_char_p, C.c_int, C.c_double]),
        "mhd_checkpoint_wait": (C.c_int, [vp]),
        "mhd_use_device": (C.c_int, [C.c_int]),
        "mhd_current_device": (C.c_int, [C.POINTER(C.c_int)]),
        "mhd_create": (C.c_int, [C.POINTER(MhdGrid), C.POINTER(MhdParams), C.POINTER(vp)]),
        "mhd_destroy": (None, [vp]),
        "mhd_upload": (C.c_int, [vp, vp, vp, vp, vp, vp]),
        "mhd_download": (C.c_int, [vp, vp, vp]),
        "mhd_setdt": (C.c_int, [vp, _PD, _PD, IP]),
        "mhd_spiral_gravity": (C.c_int, [vp, C.c_double]),
        "mhd_tvdrk": (C.c_int, [vp, C.c_double, C.c_double, IP]),
        "mhd_step": (C.c_int, [vp, _PD, _PD, _PD, IP]),
        "mhd_run": (C.c_int, [vp, C.c_int, _PD]),
        "mhd_diagnostics": (C.c_int, [vp, C.POINTER(MhdDiag)]),
        "mhd_stream": (vp, [vp]),
        "mhd_dbg_limiter": (C.c_int, [vp, C.c_int, C.c_double, DP, DP]),
        "mhd_dbg_flux": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, DP]),
        "mhd_dbg_source": (C.c_int, [vp, DP]),
        "mhd_dbg_gravity": (C.c_int, [vp, DP]),
        "mhd_batch_create": (C.c_int, [C.c_int, C.POINTER(MhdGrid), C.POINTER(MhdParams),
                                       C.POINTER(vp)]),
        "mhd_batch_destroy": (None, [vp]),
        "mhd_batch_upload": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp]),
        "mhd_batch_download": (C.c_int, [vp, C.c_int, vp, vp]),
        "mhd_batch_step": (C.c_int, [vp, C.c_int, DP, IP]),
        "mhd_batch_tune": (C.c_int, [vp, IP]),
        "mhd_batch_set_mode": (C.c_int, [vp, C.c_int, C.c_int]),
        "mhd_batch_debug_stall": (C.c_int, [vp, C.c_int, C.c_int]),
        "mhd_upload_state": (C.c_int, [vp, vp, vp]),
        "mhd_prof_enable": (C.c_int, [vp, C.c_int]),
        "mhd_set_stage_shape": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
        "mhd_set_update_path": (C.c_int, [vp, C.c_int]),
        "mhd_update_path": (C.c_int, [vp]),
        "mhd_set_state_rounding": (C.c_int, [vp, C.c_int]),
        "mhd_prof_read": (C.c_int, [vp, DP, np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")]),
        "mhd_launch_count": (C.c_longlong, [vp]),
        "mhd_timer_start": (C.c_int, [vp]),
        "mhd_timer_stop": (C.c_int, [vp, _PD]),
        "mhd_pin": (C.c_int, [vp, C.c_size_t, C.c_int]),
        "mhd_setdt_noalloc": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                        C.c_int, vp, _PD, _PD, IP]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class MhdError(RuntimeError):
    def __init__(self, code, what=""):
        msg = lib().mhd_errstr(code).decode()
        super().__init__("%s: %s (%d)" % (what, msg, code))
        self.code = code


def check(code, what=""):
    if code != MHD_OK:
        raise MhdError(code, what)
    return code


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------------------
# parameters and grids
# ---------------------------------------------------------------------------

def default_params(**over):
    """The reference's defaults (input.h, constant.h), with overrides."""
    p = MhdParams()
    lib().mhd_params_default(C.byref(p))
    for k, v in over.items():
        if k in ("limiter",) and isinstance(v, str):
            v = LIMITER[v]
        if k in ("solver",) and isinstance(v, str):
            v = SOLVER[v]
        if k in ("precision",) and isinstance(v, str):
            v = PREC[v]
        if k in ("source",) and isinstance(v, str):
            v = SOURCE[v]
        setattr(p, k, v)
    return p


class Grid:
    """A built cylindrical grid (compact j-independent tables) and its arrays."""

    def __init__(self, spec):
        self.spec = spec
        n = lib().mhd_grid_storage(C.byref(spec))
        self.storage = np.zeros(int(n))
        self.g = MhdGrid()
        check(lib().mhd_grid_build(C.byref(spec), self.storage, C.byref(self.g)), "mhd_grid_build")
        self.ix, self.jy, self.kz = spec.ix, spec.jy, spec.kz
        self.ixmax, self.jymax, self.kzmax = self.ix + 2, self.jy + 2, self.kz + 2
        self.cell = (self.ixmax, self.jymax, self.kzmax)
        self.face = (self.ixmax - 1, self.jymax - 1, self.kzmax - 1)
        self.irin = self.g.irin
        self._grav = None

    @classmethod
    def disc(cls, nr, nphi, nz):
        s = MhdGridSpec()
        check(lib().mhd_gridspec_disc(nr, nphi, nz, C.byref(s)), "mhd_gridspec_disc")
        return cls(s)

    @classmethod
    def shipped(cls, nr=None, nphi=None, nz=None):
        """The reference's stretched grid (input.h:45-76: 240x64x200); other
        cell counts keep its spacing and stretching rules."""
        s = MhdGridSpec()
        check(lib().mhd_gridspec_shipped(C.byref(s)), "mhd_gridspec_shipped")
        if nr:
            s.ix = nr
        if nphi:
            s.jy = nphi
        if nz:
            s.kz = nz
        return cls(s)

    def arr(self, name, n):
        p = getattr(self.g, name)
        return np.ctypeslib.as_array(p, shape=(n,)).copy()

    def set_initial_gravity(self):
        """Axisymmetric gravity of initialgravity.h (compact [ixmax][kzmax] tables)."""
        shp = (self.ixmax * self.kzmax,)
        gx, gy, gz = np.zeros(shp), np.zeros(shp), np.zeros(shp)
        check(lib().mhd_initial_gravity(C.byref(self.g), gx, gy, gz), "mhd_initial_gravity")
        self._grav = (gx, gy, gz)
        self.g.Grxaxi = gx.ctypes.data_as(_PD)
        self.g.Gryaxi = gy.ctypes.data_as(_PD)
        self.g.Grzaxi = gz.ctypes.data_as(_PD)

    def gravity_axi_cells(self):
        """Gr*axi expanded to the reference's [3][ixmax][jymax][kzmax] layout."""
        out = np.zeros((3,) + self.cell)
        if self._grav is not None:
            for n in range(3):
                out[n] = self._grav[n].reshape(self.ixmax, 1, self.kzmax)
        return out

    def ic_galactic_disc3(self, params):
        """GalacticDisc3 (mhd_ic_galactic_disc3): U, V, Uinit, Vinit, rhofloor."""
        shp = (9,) + self.cell
        U, V, Ui, Vi, rf = np.zeros(shp), np.zeros(shp), np.zeros(shp), np.zeros(shp), np.zeros(self.cell)
        check(lib().mhd_ic_galactic_disc3(C.byref(self.g), C.byref(params), _ptr(U), _ptr(V), _ptr(Ui), _ptr(Vi),
                                          _ptr(rf)), "mhd_ic_galactic_disc3")
        return U, V, Ui, Vi, rf

    def ic_disc(self, beta, amp=0.01, seed=0, rhocr=1.0e-4):
        U = np.zeros((9,) + self.cell)
        V = np.zeros((9,) + self.cell)
        check(lib().mhd_ic_disc(C.byref(self.g), beta, amp, seed, rhocr, _ptr(U), _ptr(V),
                                None, None, None), "mhd_ic_disc")
        return U, V


# ---------------------------------------------------------------------------
# the workloads (seeded synthetic stand-ins for the benchmark configurations)
# ---------------------------------------------------------------------------

def workload(name, nr=None, nphi=None, nz=None, **over):
    """Grid, params and initial-condition arguments of a named workload.

    disc1  64x64x32  FP64, HLLD, minmod, RK3, CFL 0.4, beta 10, gravity and cooling off
    disc2  256x256x128 FP64, HLLD, MC, RK3, beta 1, spiral (2 arms, 15 deg, 3%,
           pattern speed 0.5) + axisymmetric gravity, cooling on
    disc3  256x256x128 disc1 physics in the FP32 + FP64-repair form
    disc5  512x512x256 beta 1, cooling on, HLLD (or HLL), FP64 or FP32 form
    Shared: prcr = 1e-3 (below the disc's p/rho = 0.01), rhocr = 1e-4, betacr = 0.1,
    omegasp = 0 (inertial frame), the reference's tausp ramp.
    """
    base = dict(limiter="minmod", solver="hlld", scheme=3, cooling=0, gravity=0,
                precision="fp64", prcr=1.0e-3, rhocr=1.0e-4, betacr=0.1, cfl=0.4,
                omegasp=0.0)
    if name == "disc1":
        dims, beta = (64, 64, 32), 10.0
    elif name == "disc2":
        dims, beta = (256, 256, 128), 1.0
        base.update(limiter="mc", gravity=1, cooling=1, epssp0=0.03, omegapattern=0.5,
                    pitch=15.0 * np.pi / 180.0, armnum=2)
    elif name == "disc3":
        dims, beta = (256, 256, 128), 10.0
        base.update(precision="fp32")
    elif name == "disc5":
        dims, beta = (512, 512, 256), 1.0
        base.update(cooling=1)
    else:
        raise ValueError(name)
    dims = (nr or dims[0], nphi or dims[1], nz or dims[2])
    beta = over.pop("beta", beta)
    base.update(over)
    params = default_params(**base)
    return dims, params, dict(beta=beta, amp=0.01, seed=0)


def oracle_params(params):
    """mhd_params -> the dict the oracle wrappers take."""
    d = params.as_dict()
    d["armnum"] = float(d["armnum"])
    return d


# ---------------------------------------------------------------------------
# device context
# ---------------------------------------------------------------------------

def _path(root):
    return os.fsencode(str(root))


def binary_output(root, nout, t, grid, V):
    """BinaryOutput() of V into <root>/<nout>/ (mhd_binary_output)."""
    V = np.ascontiguousarray(V, dtype=np.float64)
    check(lib().mhd_binary_output(_path(root), int(nout), float(t), C.byref(grid.g), V), "mhd_binary_output")


def text_output(root, nout, nstep, t, grid, U, V):
    """GNUOutputCylinder + GDLOutputCylinder files under root."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    V = np.ascontiguousarray(V, dtype=np.float64)
    check(lib().mhd_gnu_output_cylinder(_path(root), int(nout), int(nstep), float(t), C.byref(grid.g), U, V),
          "mhd_gnu_output_cylinder")
    check(lib().mhd_gdl_output_cylinder(_path(root), int(nout), C.byref(grid.g), V), "mhd_gdl_output_cylinder")


def restart_read(root, num, grid):
    """V from the files of <root>/<num>/ (mhd_restart_read)."""
    V = np.zeros((9,) + grid.cell)
    check(lib().mhd_restart_read(_path(root), int(num), grid.ix, grid.jy, grid.kz, V), "mhd_restart_read")
    return V


def vtou(grid, V):
    U = np.zeros((9,) + grid.cell)
    check(lib().mhd_vtou(C.byref(grid.g), np.ascontiguousarray(V, dtype=np.float64), U), "mhd_vtou")
    return U


def check_floors(grid, params, U, V, rhofloor):
    """Check() in place on U, V; returns the three floor counters."""
    cnt = np.zeros(3, dtype=np.int32)
    check(lib().mhd_check(C.byref(grid.g), C.byref(params), U, V, np.ascontiguousarray(rhofloor), _ptr(cnt)),
          "mhd_check")
    return cnt


def restart(root, nout, tint, grid, params):
    """The reference's restart sequence (mhd_restart): returns
    U, V, Uinit, Vinit, rhofloor, t, tout."""
    shp = (9,) + grid.cell
    U, V, Ui, Vi, rf = np.zeros(shp), np.zeros(shp), np.zeros(shp), np.zeros(shp), np.zeros(grid.cell)
    t, tout = C.c_double(), C.c_double()
    check(lib().mhd_restart(_path(root), int(nout), float(tint), C.byref(grid.g), C.byref(params),
                            U, V, Ui, Vi, rf, C.byref(t), C.byref(tout)), "mhd_restart")
    return U, V, Ui, Vi, rf, t.value, tout.value


def use_device(ordinal):
    """Make CUDA device `ordinal` current for this thread (mhd_use_device):
    one process per GPU calls it with its local rank before any context."""
    check(lib().mhd_use_device(int(ordinal)), "mhd_use_device")


def current_device():
    d = C.c_int(-1)
    check(lib().mhd_current_device(C.byref(d)), "mhd_current_device")
    return d.value


class Disc:
    """One disc on the GPU: a thin wrapper over mhd_create/mhd_step/... ."""

    def __init__(self, grid, params):
        self.grid = grid
        self.params = params
        h = C.c_void_p()
        check(lib().mhd_create(C.byref(grid.g), C.byref(params), C.byref(h)), "mhd_create")
        self.h = h
        self.cell = grid.cell
        self.face = grid.face

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().mhd_destroy(self.h)
            self.h = C.c_void_p()

    __del__ = close

    def upload(self, U, V, Uinit=None, Vinit=None, rhofloor=None):
        a = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
             for x in (U, V, Uinit, Vinit, rhofloor)]
        check(lib().mhd_upload(self.h, *[_ptr(x) for x in a]), "mhd_upload")

    def download(self):
        U = np.zeros((9,) + self.cell)
        V = np.zeros((9,) + self.cell)
        check(lib().mhd_download(self.h, _ptr(U), _ptr(V)), "mhd_download")
        return U, V

    def setdt(self):
        dt, ch = C.c_double(), C.c_double()
        ijk = np.zeros(3, dtype=np.int32)
        check(lib().mhd_setdt(self.h, C.byref(dt), C.byref(ch), ijk), "mhd_setdt")
        return dt.value, ch.value, tuple(int(v) for v in ijk)

    def spiral(self, t):
        check(lib().mhd_spiral_gravity(self.h, float(t)), "mhd_spiral_gravity")

    def tvdrk(self, dt, ch):
        cnt = np.zeros(3, dtype=np.int32)
        check(lib().mhd_tvdrk(self.h, dt, ch, cnt), "mhd_tvdrk")
        return cnt

    def step(self, t):
        tt, dt, ch = C.c_double(t), C.c_double(), C.c_double()
        cnt = np.zeros(3, dtype=np.int32)
        rc = lib().mhd_step(self.h, C.byref(tt), C.byref(dt), C.byref(ch), cnt)
        if rc not in (MHD_OK, MHD_ERR_DT):
            check(rc, "mhd_step")
        return rc, tt.value, dt.value, ch.value, cnt

    def run(self, nsteps, t):
        tt = C.c_double(t)
        check(lib().mhd_run(self.h, int(nsteps), C.byref(tt)), "mhd_run")
        return tt.value

    def limiter(self, d, dt):
        Vl = np.zeros((9,) + self.face)
        Vr = np.zeros((9,) + self.face)
        check(lib().mhd_dbg_limiter(self.h, d, dt, Vl, Vr), "mhd_dbg_limiter")
        return Vl, Vr

    def flux(self, d, dt, ch):
        F = np.zeros((9,) + self.face)
        check(lib().mhd_dbg_flux(self.h, d, dt, ch, F), "mhd_dbg_flux")
        return F

    def source(self):
        S = np.zeros((9,) + self.cell)
        check(lib().mhd_dbg_source(self.h, S), "mhd_dbg_source")
        return S

    def gravity(self):
        g = np.zeros((3,) + self.cell)
        check(lib().mhd_dbg_gravity(self.h, g), "mhd_dbg_gravity")
        return g

    def diagnostics(self):
        d = MhdDiag()
        check(lib().mhd_diagnostics(self.h, C.byref(d)), "mhd_diagnostics")
        return {f: getattr(d, f) for f, _ in d._fields_}

    def stream(self):
        return lib().mhd_stream(self.h)

    def upload_state(self, U, V):
        check(lib().mhd_upload_state(self.h, _ptr(U), _ptr(V)), "mhd_upload_state")

    def download_into(self, U, V):
        check(lib().mhd_download(self.h, _ptr(U), _ptr(V)), "mhd_download")

    PROF_KINDS = ["flux_r", "flux_phi", "flux_z", "update", "ghost", "setdt", "trig", "convert", "stage",
                  "zupdate"]

    def prof(self, on=True):
        check(lib().mhd_prof_enable(self.h, 1 if on else 0), "mhd_prof_enable")

    def prof_read(self):
        ms = np.zeros(len(self.PROF_KINDS))
        n = np.zeros(len(self.PROF_KINDS), dtype=np.int64)
        check(lib().mhd_prof_read(self.h, ms, n), "mhd_prof_read")
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(self.PROF_KINDS)}

    def checkpoint_begin(self, root, nout, t):
        """Asynchronous BinaryOutput of the current V (mhd_checkpoint_begin)."""
        check(lib().mhd_checkpoint_begin(self.h, _path(root), int(nout), float(t)), "mhd_checkpoint_begin")

    def checkpoint_wait(self):
        check(lib().mhd_checkpoint_wait(self.h), "mhd_checkpoint_wait")

    def set_stage_shape(self, fused=True, tj=7, seg=32):
        """fused: 0/False split kernels, 1/True one fused stage kernel (tj = 7
        j-cells per tile, seg r-cells per run), 2 z fluxes fused into the
        update (mhd_set_stage_shape)."""
        check(lib().mhd_set_stage_shape(self.h, int(fused), int(tj), int(seg)), "mhd_set_stage_shape")

    def set_update_path(self, tma):
        """1: the split stage's update stages its tiles in shared memory with
        tensor copies; 0: thread-by-thread loads (mhd_set_update_path)."""
        check(lib().mhd_set_update_path(self.h, int(tma)), "mhd_set_update_path")

    def set_state_rounding(self, on=True):
        """Plain form only: FP64 arithmetic, U and V stored rounded to FP32 after
        every stage -- the FP32-storage error floor (mhd_set_state_rounding)."""
        check(lib().mhd_set_state_rounding(self.h, 1 if on else 0), "mhd_set_state_rounding")

    def update_path(self):
        return int(lib().mhd_update_path(self.h))

    def launches(self):
        return int(lib().mhd_launch_count(self.h))

    def timer_start(self):
        check(lib().mhd_timer_start(self.h), "mhd_timer_start")

    def timer_stop(self):
        ms = C.c_double()
        check(lib().mhd_timer_stop(self.h, C.byref(ms)), "mhd_timer_stop")
        return ms.value


def pin(a, on=True):
    """page-lock a numpy array's buffer for fast async copies"""
    check(lib().mhd_pin(_ptr(a), a.nbytes, 1 if on else 0), "mhd_pin")


# ---------------------------------------------------------------------------
# batched discs
# ---------------------------------------------------------------------------

class Batch:
    """Many independent discs stepped together (mhd_batch_*)."""

    def __init__(self, grids, params):
        self.grids = list(grids)
        n = len(self.grids)
        G = (MhdGrid * n)(*[g.g for g in self.grids])
        Pp = (MhdParams * n)(*params)
        h = C.c_void_p()
        check(lib().mhd_batch_create(n, G, Pp, C.byref(h)), "mhd_batch_create")
        self.h = h
        self.n = n

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().mhd_batch_destroy(self.h)
            self.h = C.c_void_p()

    __del__ = close

    def upload(self, d, U, V):
        U = np.ascontiguousarray(U, dtype=np.float64)
        V = np.ascontiguousarray(V, dtype=np.float64)
        check(lib().mhd_batch_upload(self.h, d, _ptr(U), _ptr(V), None, None, None), "mhd_batch_upload")

    def download(self, d):
        g = self.grids[d]
        U = np.zeros((9,) + g.cell)
        V = np.zeros((9,) + g.cell)
        check(lib().mhd_batch_download(self.h, d, _ptr(U), _ptr(V)), "mhd_batch_download")
        return U, V

    def step(self, nsteps, t):
        t = np.array(t, dtype=np.float64, copy=True)   # advanced in place by the library
        st = np.zeros(self.n, dtype=np.int32)
        check(lib().mhd_batch_step(self.h, int(nsteps), t, st), "mhd_batch_step")
        return t, st

    def tune(self):
        best = np.zeros(5, dtype=np.int32)
        check(lib().mhd_batch_tune(self.h, best), "mhd_batch_tune")
        return tuple(int(v) for v in best)

    def debug_stall(self, disc, spin_limit=4096):
        check(lib().mhd_batch_debug_stall(self.h, int(disc), int(spin_limit)), "mhd_batch_debug_stall")

    def set_mode(self, mode, arg=0):
        """0 persistent (tile candidate arg), 1 phased, 2 disc graph on arg branches."""
        check(lib().mhd_batch_set_mode(self.h, int(mode), int(arg)), "mhd_batch_set_mode")


def batch_workload(n=64, seed=7):
    """The batched workload: n discs with sizes drawn from seed 7 (nr in
    {32,64,96,128}, nphi in {64,128,256}, nz in {32,48,64}), beta log-uniform in
    [1,100], spiral amplitude uniform in [0, 0.05], pattern speed uniform in
    [0.3, 0.8], per-disc perturbation seed; precision form, HLLD, minmod, RK3,
    spiral + axisymmetric gravity on, cooling on."""
    rng = np.random.default_rng(seed)
    out = []
    for d in range(n):
        nr = int(rng.choice([32, 64, 96, 128]))
        nphi = int(rng.choice([64, 128, 256]))
        nz = int(rng.choice([32, 48, 64]))
        beta = float(10 ** rng.uniform(0.0, 2.0))
        eps = float(rng.uniform(0.0, 0.05))
        omp = float(rng.uniform(0.3, 0.8))
        (nr, nphi, nz), params, ic = workload("disc2", nr=nr, nphi=nphi, nz=nz, limiter="minmod",
                                              precision="fp32", epssp0=eps, omegapattern=omp, beta=beta)
        ic["seed"] = 1000 + d
        out.append(((nr, nphi, nz), params, ic))
    return out

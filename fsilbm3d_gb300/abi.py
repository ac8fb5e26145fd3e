"""ctypes binding of libfsi_gpu.so (include/fsi_gpu.h).

Block mirrors the reference's LBMBlock (FluidDomain.f90:17-56) and the
routines the hot path calls on it; every method is one C-ABI call. Arrays
cross the boundary in the reference's Fortran layout: fIn(z,y,x,0:18) is a
numpy array of shape (19, xDim, yDim, zDim) in C order (the same memory).
Errors come back as FsiError carrying the ABI status code and message, in
place of the reference's `stop`.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

FSI_OK = 0
FSI_E_ARG, FSI_E_CUDA, FSI_E_NAN, FSI_E_TIMEOUT, FSI_E_BC, FSI_E_RANGE, FSI_E_STATE = -1, -2, -3, -4, -5, -6, -7
PREC_F64, PREC_F64_FAST, PREC_F32, PREC_F16, PREC_BF16 = 0, 1, 2, 3, 4
PRECISIONS = {"f64": PREC_F64, "f64_fast": PREC_F64_FAST, "f32": PREC_F32, "f16": PREC_F16, "bf16": PREC_BF16}
_STORE_BYTES = {PREC_F64: 8, PREC_F64_FAST: 8, PREC_F32: 4, PREC_F16: 2, PREC_BF16: 2}

DP = C.POINTER(C.c_double)


class FsiError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("fsi error %d: %s" % (code, msg))
        self.code = code


class BlockDesc(C.Structure):
    _fields_ = [
        ("xDim", C.c_int), ("yDim", C.c_int), ("zDim", C.c_int),
        ("dh", C.c_double), ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double),
        ("bndConds", C.c_int * 6),
        ("iCollidModel", C.c_int),
        ("nu", C.c_double),
        ("m_collid", DP), ("m_force", DP),
        ("precision", C.c_int),
        ("denIn", C.c_double),
        ("uvwIn", C.c_double * 3),
        ("shearRateIn", C.c_double * 3),
        ("velocityKind", C.c_int),
    ]


_lib = None

# every symbol the header declares
SYMBOLS = [
    "fsi_last_error", "fsi_device_info", "fsi_block_create", "fsi_block_destroy", "fsi_block_get_params",
    "fsi_block_upload_f", "fsi_block_download_f", "fsi_block_initialise", "fsi_block_set_boundary_conditions",
    "fsi_block_macro", "fsi_block_step", "fsi_block_run", "fsi_ib_set_bodies", "fsi_ib_solve",
    "fsi_ib_get_stencil", "fsi_ib_get_window", "fsi_pair_create", "fsi_pair_destroy", "fsi_pair_extract",
    "fsi_pair_father_to_son", "fsi_pair_son_to_father", "fsi_pair_father_to_son_static",
]
# son face cells the allocation-free father-to-son variant can hold
STATIC_FACE_CELLS = 65536


def library_path():
    return os.path.join(HERE, "libfsi_gpu.so")


def load_library():
    """Load libfsi_gpu.so and declare argument types. Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise FsiError(FSI_E_STATE, "libfsi_gpu.so not built: run __graft_entry__.build() "
                                    "or python fsilbm3d_gb300/build.py")
    L = C.CDLL(path)
    VP = C.c_void_p
    IP = C.POINTER(C.c_int)
    L.fsi_last_error.argtypes = [C.c_char_p, C.c_int]
    L.fsi_device_info.argtypes = [IP, IP, IP]
    L.fsi_block_create.argtypes = [C.POINTER(VP), C.POINTER(BlockDesc)]
    L.fsi_block_destroy.argtypes = [VP]
    L.fsi_block_get_params.argtypes = [VP, DP, DP, DP, DP]
    L.fsi_block_upload_f.argtypes = [VP, DP]
    L.fsi_block_download_f.argtypes = [VP, DP]
    L.fsi_block_initialise.argtypes = [VP, C.c_double]
    L.fsi_block_set_boundary_conditions.argtypes = [VP, C.c_double]
    L.fsi_block_macro.argtypes = [VP, DP, DP, DP]
    L.fsi_block_step.argtypes = [VP, DP, C.c_double]
    L.fsi_block_run.argtypes = [VP, DP, C.c_double, C.c_int, C.POINTER(C.c_float)]
    L.fsi_ib_set_bodies.argtypes = [VP, C.c_int, IP, IP]
    L.fsi_ib_solve.argtypes = [VP, DP, DP, DP, DP, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                               DP, IP, DP]
    L.fsi_ib_get_stencil.argtypes = [VP, C.POINTER(C.c_int16), C.POINTER(C.c_float)]
    L.fsi_ib_get_window.argtypes = [VP, IP]
    L.fsi_pair_create.argtypes = [C.POINTER(VP), VP, VP, C.c_int]
    L.fsi_pair_destroy.argtypes = [VP]
    L.fsi_pair_extract.argtypes = [VP, C.c_int]
    L.fsi_pair_father_to_son.argtypes = [VP, C.c_int, DP]
    L.fsi_pair_son_to_father.argtypes = [VP, DP]
    L.fsi_pair_father_to_son_static.argtypes = [VP, C.c_int, DP]
    for s in SYMBOLS:
        getattr(L, s).restype = C.c_int
    _lib = L
    return L


lib = load_library


def _check(rc):
    if rc != FSI_OK:
        buf = C.create_string_buffer(1024)
        load_library().fsi_last_error(buf, 1024)
        raise FsiError(rc, buf.value.decode(errors="replace"))


def _dp(a):
    return a.ctypes.data_as(DP)


def _vec3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))


def device_info():
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _check(load_library().fsi_device_info(C.byref(sm), C.byref(ma), C.byref(mi)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value)}


class Block:
    """One LBM block on the GPU (LBMBlock, FluidDomain.f90:17-56)."""

    def __init__(self, xDim, yDim, zDim, dh=1.0, origin=(0.0, 0.0, 0.0), bndConds=(301,) * 6, iCollidModel=1,
                 nu=0.1 / 3.0, precision=PREC_F64, denIn=1.0, uvwIn=(0.0, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.0),
                 velocityKind=0, m_collid=None, m_force=None):
        L = load_library()
        d = BlockDesc()
        d.xDim, d.yDim, d.zDim = int(xDim), int(yDim), int(zDim)
        d.dh = dh
        d.xmin, d.ymin, d.zmin = origin
        d.bndConds[:] = [int(c) for c in bndConds]
        d.iCollidModel = int(iCollidModel)
        d.nu = nu
        self._mats = None
        if m_collid is not None and m_force is not None:
            self._mats = (np.asfortranarray(m_collid, dtype=np.float64).ravel(order="F").copy(),
                          np.asfortranarray(m_force, dtype=np.float64).ravel(order="F").copy())
            d.m_collid, d.m_force = _dp(self._mats[0]), _dp(self._mats[1])
        d.precision = int(precision)
        d.denIn = denIn
        d.uvwIn[:] = list(uvwIn)
        d.shearRateIn[:] = list(shearRateIn)
        d.velocityKind = int(velocityKind)
        self.desc = d
        self.dims = (int(xDim), int(yDim), int(zDim))
        self.N = int(xDim) * int(yDim) * int(zDim)
        self.dh = dh
        self.precision = int(precision)
        h = C.c_void_p()
        _check(L.fsi_block_create(C.byref(h), C.byref(d)))
        self.h = h
        self.nbodies = 0
        self.Mtot = 0

    def close(self):
        if getattr(self, "h", None):
            load_library().fsi_block_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def store_bytes(self):
        return _STORE_BYTES[self.precision]

    def params(self):
        tau, om = C.c_double(), C.c_double()
        mc = np.zeros(361)
        mf = np.zeros(361)
        _check(load_library().fsi_block_get_params(self.h, C.byref(tau), C.byref(om), _dp(mc), _dp(mf)))
        return tau.value, om.value, mc.reshape(19, 19, order="F"), mf.reshape(19, 19, order="F")

    # -- state transfer (write_continue_/read_continue_ layout) --
    def upload_f(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.size != 19 * self.N:
            raise ValueError("fIn must hold 19*xDim*yDim*zDim values")
        _check(load_library().fsi_block_upload_f(self.h, _dp(f)))

    def download_f(self, out=None):
        X, Y, Z = self.dims
        if out is None:
            out = np.empty((19, X, Y, Z))
        _check(load_library().fsi_block_download_f(self.h, _dp(out)))
        return out

    # -- the reference's block routines --
    def initialise(self, time=0.0):
        """initialise_flow (FluidDomain.f90:524-544)"""
        _check(load_library().fsi_block_initialise(self.h, time))

    def set_boundary_conditions(self, blktime=0.0):
        """set_boundary_conditions_ (FluidDomain.f90:616-1126)"""
        _check(load_library().fsi_block_set_boundary_conditions(self.h, blktime))

    def calculate_macro_quantities(self, volumeForce=(0.0, 0.0, 0.0), download=True):
        """calculate_macro_quantities_ (FluidDomain.f90:1128-1145); returns (den, uuu)
        with shapes (xDim,yDim,zDim) and (3,xDim,yDim,zDim) in C order."""
        X, Y, Z = self.dims
        vf = _vec3(volumeForce)
        if not download:
            _check(load_library().fsi_block_macro(self.h, _dp(vf), DP(), DP()))
            return None
        den = np.empty((X, Y, Z))
        uuu = np.empty((3, X, Y, Z))
        _check(load_library().fsi_block_macro(self.h, _dp(vf), _dp(den), _dp(uuu)))
        return den, uuu

    def step(self, volumeForce=(0.0, 0.0, 0.0), blktime=0.0):
        """add_volume_force_, collision_, halfwayBCset_, streaming_,
        set_boundary_conditions_ (LBMBlockComm.f90:288-303)"""
        vf = _vec3(volumeForce)
        _check(load_library().fsi_block_step(self.h, _dp(vf), blktime))

    def run(self, nsteps, volumeForce=(0.0, 0.0, 0.0), blktime0=0.0):
        """nsteps fluid steps from a captured CUDA graph; returns device ms"""
        vf = _vec3(volumeForce)
        ms = C.c_float()
        _check(load_library().fsi_block_run(self.h, _dp(vf), blktime0, int(nsteps), C.byref(ms)))
        return ms.value

    # -- immersed boundary (Solidbody.f90) --
    def ib_set_bodies(self, M, bc=None):
        M = np.ascontiguousarray(M, dtype=np.int32)
        bcs = None if bc is None else np.ascontiguousarray(bc, dtype=np.int32)
        IP = C.POINTER(C.c_int)
        _check(load_library().fsi_ib_set_bodies(self.h, int(M.size), M.ctypes.data_as(IP),
                                                bcs.ctypes.data_as(IP) if bcs is not None else IP()))
        self.nbodies = int(M.size)
        self.Mtot = int(M.sum())

    def ib_solve(self, xyz, vel, area, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, dt=None, Uref=1.0, ntol=3,
                 dtol=1e-5, eforce=None):
        """calculate_interaction_force (Solidbody.f90:869-918) for the block's
        bodies; returns (eforce (Mtot,3), iterations, residual)"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        if area.size != self.Mtot or xyz.size != 3 * self.Mtot or vel.size != 3 * self.Mtot:
            raise ValueError("marker arrays do not match the bodies set with ib_set_bodies")
        if eforce is None:
            eforce = np.empty(3 * self.Mtot)
        vf = _vec3(volumeForce)
        it = C.c_int()
        res = C.c_double()
        _check(load_library().fsi_ib_solve(self.h, _dp(xyz), _dp(vel), _dp(area), _dp(vf), denIn,
                                           self.dh if dt is None else dt, Uref, int(ntol), dtol,
                                           _dp(eforce), C.byref(it), C.byref(res)))
        return eforce.reshape(-1, 3), it.value, res.value

    def ib_stencil(self):
        ei = np.empty(12 * self.Mtot, dtype=np.int16)
        ew = np.empty(12 * self.Mtot, dtype=np.float32)
        _check(load_library().fsi_ib_get_stencil(self.h, ei.ctypes.data_as(C.POINTER(C.c_int16)),
                                                 ew.ctypes.data_as(C.POINTER(C.c_float))))
        return ei.reshape(-1, 12), ew.reshape(-1, 12)

    def ib_window(self):
        box = (C.c_int * 6)()
        _check(load_library().fsi_ib_get_window(self.h, box))
        return tuple(box)


class Pair:
    """A father/son block pair (CommPair, LBMBlockComm.f90:11-18)."""

    def __init__(self, father, son, scheme=1):
        h = C.c_void_p()
        _check(load_library().fsi_pair_create(C.byref(h), father.h, son.h, int(scheme)))
        self.h = h
        self.father, self.son = father, son

    def close(self):
        if getattr(self, "h", None):
            load_library().fsi_pair_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def extract(self, time_level):
        """extract_interpolate_layer (LBMBlockComm.f90:340-505)"""
        _check(load_library().fsi_pair_extract(self.h, int(time_level)))

    def father_to_son(self, n_timeStep, volumeForce=(0.0, 0.0, 0.0)):
        """interpolation_father_to_son (LBMBlockComm.f90:655-806)"""
        vf = _vec3(volumeForce)
        _check(load_library().fsi_pair_father_to_son(self.h, int(n_timeStep), _dp(vf)))

    def father_to_son_static(self, n_timeStep, volumeForce=(0.0, 0.0, 0.0)):
        """father_to_son without any device allocation: for hosts that may not
        allocate GPU memory inside their time loop (fsi_pair_father_to_son_static)"""
        vf = _vec3(volumeForce)
        _check(load_library().fsi_pair_father_to_son_static(self.h, int(n_timeStep), _dp(vf)))

    def son_to_father(self, volumeForce=(0.0, 0.0, 0.0)):
        """deliver_son_to_father (LBMBlockComm.f90:546-653)"""
        vf = _vec3(volumeForce)
        _check(load_library().fsi_pair_son_to_father(self.h, _dp(vf)))

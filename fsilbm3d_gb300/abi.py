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
PREC_F64, PREC_F64_FAST, PREC_F32, PREC_F16, PREC_BF16, PREC_F64_DW = 0, 1, 2, 3, 4, 5
PRECISIONS = {"f64": PREC_F64, "f64_fast": PREC_F64_FAST, "f32": PREC_F32, "f16": PREC_F16, "bf16": PREC_BF16,
              "f64_dw": PREC_F64_DW}
_STORE_BYTES = {PREC_F64: 8, PREC_F64_FAST: 8, PREC_F32: 4, PREC_F16: 2, PREC_BF16: 2, PREC_F64_DW: 8}

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
        ("params", C.c_double * 10),
    ]


_lib = None

# every symbol the header declares
SYMBOLS = [
    "fsi_last_error", "fsi_device_info", "fsi_block_create", "fsi_block_destroy", "fsi_block_get_params",
    "fsi_block_upload_f", "fsi_block_download_f", "fsi_block_initialise", "fsi_block_set_boundary_conditions",
    "fsi_block_macro", "fsi_block_step", "fsi_block_run", "fsi_ib_set_bodies", "fsi_ib_solve",
    "fsi_ib_get_stencil", "fsi_ib_get_window", "fsi_pair_create", "fsi_pair_destroy", "fsi_pair_extract",
    "fsi_pair_father_to_son", "fsi_pair_son_to_father", "fsi_pair_father_to_son_static",
    "fsi_mlp_create", "fsi_mlp_destroy", "fsi_mlp_set_params", "fsi_mlp_get_params", "fsi_mlp_set_norm",
    "fsi_mlp_forward", "fsi_mlp_grad", "fsi_mlp_train", "fsi_ib_solve_warm", "fsi_ib_solve_seeded", "fsi_block_timer",
    "fsi_block_set_kernel", "fsi_block_ib_step", "fsi_block_ib_step_async", "fsi_block_ib_wait",
    "fsi_batch_create", "fsi_batch_destroy", "fsi_batch_ib_step", "fsi_batch_tune", "fsi_batch_set_threads",
    "fsi_block_set_ib_mode", "fsi_block_pack_flow", "fsi_block_flux", "fsi_block_probes",
    "fsi_block_get_omega2", "fsi_block_get_tau_all", "fsi_continue_write", "fsi_continue_read",
]
IB_AUTO, IB_GRID, IB_CLUSTER, IB_OVERLAP, IB_GATHER = 0, 1, 2, 3, 4
KERNEL_AUTO, KERNEL_PAIRED, KERNEL_PIPELINED = 0, 1, 2
# the warm-start perceptron (FSI_MLP_* in the header)
MLP_IN, MLP_OUT, MLP_NPARAM, MLP_NNORM = 12, 3, 5187, 30
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
    L.fsi_block_get_omega2.argtypes = [VP, DP]
    L.fsi_continue_write.argtypes = [C.c_char_p, C.POINTER(VP), C.c_int, C.c_int, C.c_double]
    L.fsi_continue_read.argtypes = [C.c_char_p, C.POINTER(VP), C.c_int, C.POINTER(C.c_int), DP]
    L.fsi_block_get_tau_all.argtypes = [VP, DP]
    L.fsi_block_upload_f.argtypes = [VP, DP]
    L.fsi_block_download_f.argtypes = [VP, DP]
    L.fsi_block_initialise.argtypes = [VP, C.c_double]
    L.fsi_block_set_boundary_conditions.argtypes = [VP, C.c_double]
    L.fsi_block_macro.argtypes = [VP, DP, DP, DP]
    # the calls of a time loop take plain addresses (see _vp)
    L.fsi_block_step.argtypes = [VP, VP, C.c_double]
    L.fsi_block_run.argtypes = [VP, DP, C.c_double, C.c_int, C.POINTER(C.c_float)]
    L.fsi_block_timer.argtypes = [VP, C.c_int, C.POINTER(C.c_float)]
    L.fsi_block_set_kernel.argtypes = [VP, C.c_int]
    L.fsi_block_set_ib_mode.argtypes = [VP, C.c_int]
    L.fsi_block_pack_flow.argtypes = [VP, DP, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_float)]
    L.fsi_block_flux.argtypes = [VP, DP, C.c_double, C.c_double, DP]
    L.fsi_block_probes.argtypes = [VP, DP, C.c_int, DP, C.c_double, DP]
    L.fsi_batch_create.argtypes = [C.POINTER(VP), C.c_int, C.POINTER(VP)]
    L.fsi_batch_destroy.argtypes = [VP]
    L.fsi_batch_ib_step.argtypes = [VP, DP, DP, DP, DP, DP, DP, DP, C.c_int, C.c_double, DP, DP, IP, DP]
    L.fsi_batch_tune.argtypes = [VP, C.c_int, IP, C.POINTER(C.c_float)]
    L.fsi_batch_set_threads.argtypes = [VP, C.c_int]
    L.fsi_block_ib_step.argtypes = [VP, VP, VP, VP, VP, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double,
                                    C.c_double, VP, IP, DP]
    L.fsi_block_ib_step_async.argtypes = [VP, VP, VP, VP, VP, C.c_double, C.c_double, C.c_double, C.c_int,
                                          C.c_double, C.c_double]
    L.fsi_block_ib_wait.argtypes = [VP, VP, IP, DP]
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
    FP = C.POINTER(C.c_float)
    L.fsi_mlp_create.argtypes = [C.POINTER(VP), C.c_ulonglong]
    L.fsi_mlp_destroy.argtypes = [VP]
    L.fsi_mlp_set_params.argtypes = [VP, FP, C.c_int]
    L.fsi_mlp_get_params.argtypes = [VP, FP, C.c_int]
    L.fsi_mlp_set_norm.argtypes = [VP, FP]
    L.fsi_mlp_forward.argtypes = [VP, FP, C.c_int, FP]
    L.fsi_mlp_grad.argtypes = [VP, FP, FP, C.c_int, FP, FP]
    L.fsi_mlp_train.argtypes = [VP, FP, FP, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong, FP]
    L.fsi_ib_solve_warm.argtypes = [VP, DP, DP, DP, DP, DP, C.c_double, C.c_double, C.c_double, C.c_int,
                                    C.c_double, VP, FP, DP, IP, DP]
    L.fsi_ib_solve_seeded.argtypes = [VP, DP, DP, DP, DP, DP, C.c_double, C.c_double, C.c_double, C.c_int,
                                      C.c_double, DP, IP, DP]
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


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f32(a, cols):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, cols))


def _vec3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))


def _vp(a):
    """the address of a contiguous array, for the calls of a time loop
    (declared with void pointers): a third of the cost of a typed pointer"""
    return a.ctypes.data


def _v3(v):
    """three doubles as a ctypes array"""
    x, y, z = v
    return (C.c_double * 3)(x, y, z)


def device_info():
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _check(load_library().fsi_device_info(C.byref(sm), C.byref(ma), C.byref(mi)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value)}


class Block:
    """One LBM block on the GPU (LBMBlock, FluidDomain.f90:17-56)."""

    def __init__(self, xDim, yDim, zDim, dh=1.0, origin=(0.0, 0.0, 0.0), bndConds=(301,) * 6, iCollidModel=1,
                 nu=0.1 / 3.0, precision=PREC_F64, denIn=1.0, uvwIn=(0.0, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.0),
                 velocityKind=0, m_collid=None, m_force=None, params=None):
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
        if params is not None:
            d.params[:len(params)] = [float(v) for v in params]
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

    def omega2(self):
        """Omega2 of the TRT model (0 for the others)"""
        v = C.c_double()
        _check(load_library().fsi_block_get_omega2(self.h, C.byref(v)))
        return v.value

    def tau_all(self):
        """tau_all(z,y,x) as an array of shape (xDim, yDim, zDim)"""
        X, Y, Z = self.dims
        out = np.empty((X, Y, Z))
        _check(load_library().fsi_block_get_tau_all(self.h, _dp(out)))
        return out

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
        _check(load_library().fsi_block_step(self.h, _v3(volumeForce), blktime))

    def run(self, nsteps, volumeForce=(0.0, 0.0, 0.0), blktime0=0.0):
        """nsteps fluid steps from a captured CUDA graph; returns device ms"""
        vf = _vec3(volumeForce)
        ms = C.c_float()
        _check(load_library().fsi_block_run(self.h, _dp(vf), blktime0, int(nsteps), C.byref(ms)))
        return ms.value

    def set_kernel(self, kernel):
        """bulk step kernel of the offset forms: KERNEL_AUTO, _PAIRED, _PIPELINED"""
        _check(load_library().fsi_block_set_kernel(self.h, int(kernel)))

    # -- outputs (main.f90:107-141), packed on the GPU --
    def pack_flow(self, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, Uref=1.0, offset=0):
        """write_flow_ fields: FP32 array (4, nx, ny, nz) of p, u, v, w"""
        X, Y, Z = self.dims
        nx, ny, nz = X - 2 * offset, Y - 2 * offset, Z - 2 * offset
        out = np.empty((4, nx, ny, nz), dtype=np.float32)
        vf = _vec3(volumeForce)
        _check(load_library().fsi_block_pack_flow(self.h, _dp(vf), denIn, Uref, int(offset), _fp(out)))
        return out

    def flux(self, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, Uref=1.0):
        """write_fluid_flux: (in, mid, out) normalised x-fluxes"""
        f = np.empty(3)
        vf = _vec3(volumeForce)
        _check(load_library().fsi_block_flux(self.h, _dp(vf), denIn, Uref, _dp(f)))
        return f

    def probes(self, xyz, volumeForce=(0.0, 0.0, 0.0), Uref=1.0):
        """fluid probes: (n, 3) velocities / Uref at the points xyz (n, 3)"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = xyz.size // 3
        uvw = np.empty(3 * max(n, 1))
        vf = _vec3(volumeForce)
        _check(load_library().fsi_block_probes(self.h, _dp(vf), n, _dp(xyz), Uref, _dp(uvw)))
        return uvw[:3 * n].reshape(-1, 3)

    def set_ib_mode(self, mode):
        """IB stage of ib_step: IB_GRID (cooperative, then the step) or
        IB_CLUSTER (one cluster beside the bulk step)"""
        _check(load_library().fsi_block_set_ib_mode(self.h, int(mode)))

    def timer_start(self):
        """mark the start of a timed region on the block's stream"""
        _check(load_library().fsi_block_timer(self.h, 0, None))

    def timer_stop(self):
        """device milliseconds since timer_start (waits for the stream)"""
        ms = C.c_float()
        _check(load_library().fsi_block_timer(self.h, 1, C.byref(ms)))
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

    def ib_step(self, xyz, vel, area, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, dt=None, Uref=1.0, ntol=3, dtol=1e-5,
                blktime=0.0):
        """ib_solve then step(volumeForce, blktime) in one call; returns
        (eforce (Mtot,3), iterations, residual) while the fluid step runs"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        if area.size != self.Mtot or xyz.size != 3 * self.Mtot or vel.size != 3 * self.Mtot:
            raise ValueError("marker arrays do not match the bodies set with ib_set_bodies")
        eforce = np.empty(3 * self.Mtot)
        it = C.c_int()
        res = C.c_double()
        _check(load_library().fsi_block_ib_step(self.h, _vp(xyz), _vp(vel), _vp(area), _v3(volumeForce), denIn,
                                                self.dh if dt is None else dt, Uref, int(ntol), dtol, blktime,
                                                _vp(eforce), C.byref(it), C.byref(res)))
        return eforce.reshape(-1, 3), it.value, res.value

    def ib_step_async(self, xyz, vel, area, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, dt=None, Uref=1.0, ntol=3,
                      dtol=1e-5, blktime=0.0):
        """ib_step's first half: queues the IB stage and the fluid step and
        returns at once; ib_wait() returns (eforce (Mtot,3), iterations, residual)"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        if area.size != self.Mtot or xyz.size != 3 * self.Mtot or vel.size != 3 * self.Mtot:
            raise ValueError("marker arrays do not match the bodies set with ib_set_bodies")
        _check(load_library().fsi_block_ib_step_async(self.h, _vp(xyz), _vp(vel), _vp(area), _v3(volumeForce),
                                                      denIn, self.dh if dt is None else dt, Uref, int(ntol), dtol,
                                                      blktime))

    def ib_wait(self):
        eforce = np.empty(3 * max(self.Mtot, 1))
        it = C.c_int()
        res = C.c_double()
        _check(load_library().fsi_block_ib_wait(self.h, _vp(eforce), C.byref(it), C.byref(res)))
        return eforce[:3 * self.Mtot].reshape(-1, 3), it.value, res.value

    def ib_solve_warm(self, xyz, vel, area, aux=None, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, dt=None, Uref=1.0,
                      ntol=3, dtol=1e-5, warm=None, features=False):
        """ib_solve with the learned warm start (fast forms only).
        aux (Mtot,6): acceleration, normal per marker (None: zeros); warm: an
        Mlp or None; features=True also returns the (Mtot,12) feature array.
        Returns (eforce, iterations, residual[, features])."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        if area.size != self.Mtot or xyz.size != 3 * self.Mtot or vel.size != 3 * self.Mtot:
            raise ValueError("marker arrays do not match the bodies set with ib_set_bodies")
        auxp = DP()
        if aux is not None:
            aux = np.ascontiguousarray(aux, dtype=np.float64).reshape(-1)
            if aux.size != 6 * self.Mtot:
                raise ValueError("aux must hold 6 values per marker")
            auxp = _dp(aux)
        eforce = np.empty(3 * self.Mtot)
        feat = np.empty((self.Mtot, MLP_IN), dtype=np.float32) if features else None
        vf = _vec3(volumeForce)
        it = C.c_int()
        res = C.c_double()
        _check(load_library().fsi_ib_solve_warm(self.h, _dp(xyz), _dp(vel), _dp(area), auxp, _dp(vf), denIn,
                                                self.dh if dt is None else dt, Uref, int(ntol), dtol,
                                                warm.h if warm is not None else None,
                                                _fp(feat) if features else C.POINTER(C.c_float)(),
                                                _dp(eforce), C.byref(it), C.byref(res)))
        out = (eforce.reshape(-1, 3), it.value, res.value)
        return out + (feat,) if features else out

    def ib_solve_seeded(self, xyz, vel, area, guess, volumeForce=(0.0, 0.0, 0.0), denIn=1.0, dt=None, Uref=1.0,
                        ntol=3, dtol=1e-5):
        """ib_solve started from guess (Mtot,3), e.g. the previous step's
        Lagrangian force (fast forms only); returns (eforce, iterations, residual)"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        guess = np.ascontiguousarray(guess, dtype=np.float64).reshape(-1)
        if area.size != self.Mtot or xyz.size != 3 * self.Mtot or vel.size != 3 * self.Mtot or \
                guess.size != 3 * self.Mtot:
            raise ValueError("marker arrays do not match the bodies set with ib_set_bodies")
        eforce = np.empty(3 * self.Mtot)
        vf = _vec3(volumeForce)
        it = C.c_int()
        res = C.c_double()
        _check(load_library().fsi_ib_solve_seeded(self.h, _dp(xyz), _dp(vel), _dp(area), _dp(guess), _dp(vf), denIn,
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


class Mlp:
    """The warm-start perceptron (12 -> 64 -> 64 -> 3, tanh, FP32) on the
    current device: inference, full-batch gradient and Adam training run in
    the library's CUDA kernels."""

    def __init__(self, seed=0):
        L = load_library()
        h = C.c_void_p()
        _check(L.fsi_mlp_create(C.byref(h), C.c_ulonglong(seed)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load_library().fsi_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        P = np.empty(MLP_NPARAM, dtype=np.float32)
        _check(load_library().fsi_mlp_get_params(self.h, _fp(P), MLP_NPARAM))
        return P

    @params.setter
    def params(self, P):
        P = np.ascontiguousarray(P, dtype=np.float32).reshape(-1)
        _check(load_library().fsi_mlp_set_params(self.h, _fp(P), int(P.size)))

    def set_norm(self, mean_in, std_in, mean_out, std_out):
        nrm = np.concatenate([np.ravel(mean_in), np.ravel(std_in), np.ravel(mean_out), np.ravel(std_out)])
        nrm = np.ascontiguousarray(nrm, dtype=np.float32)
        if nrm.size != MLP_NNORM:
            raise ValueError("expected %d statistics" % MLP_NNORM)
        _check(load_library().fsi_mlp_set_norm(self.h, _fp(nrm)))

    def fit_norm(self, X, Y, floor=1e-6):
        """statistics from a training set (deviations floored at floor)"""
        X = np.asarray(X, dtype=np.float64).reshape(-1, MLP_IN)
        Y = np.asarray(Y, dtype=np.float64).reshape(-1, MLP_OUT)
        self.set_norm(X.mean(0), np.maximum(X.std(0), floor), Y.mean(0), np.maximum(Y.std(0), floor))

    def forward(self, X):
        X = _f32(X, MLP_IN)
        Y = np.empty((X.shape[0], MLP_OUT), dtype=np.float32)
        _check(load_library().fsi_mlp_forward(self.h, _fp(X), int(X.shape[0]), _fp(Y)))
        return Y

    def grad(self, X, Y):
        X, Y = _f32(X, MLP_IN), _f32(Y, MLP_OUT)
        if X.shape[0] != Y.shape[0]:
            raise ValueError("X and Y hold different sample counts")
        g = np.empty(MLP_NPARAM, dtype=np.float32)
        loss = C.c_float()
        _check(load_library().fsi_mlp_grad(self.h, _fp(X), _fp(Y), int(X.shape[0]), _fp(g), C.byref(loss)))
        return g, loss.value

    def train(self, X, Y, epochs=100, batch=256, lr=1e-3, seed=0):
        """Adam over shuffled mini-batches; returns the per-epoch mean loss"""
        X, Y = _f32(X, MLP_IN), _f32(Y, MLP_OUT)
        if X.shape[0] != Y.shape[0]:
            raise ValueError("X and Y hold different sample counts")
        hist = np.empty(int(epochs), dtype=np.float32)
        _check(load_library().fsi_mlp_train(self.h, _fp(X), _fp(Y), int(X.shape[0]), int(epochs), int(batch),
                                            C.c_float(lr), C.c_ulonglong(seed), _fp(hist)))
        return hist


class Batch:
    """Many independent blocks stepped together (one CUDA graph per step):
    each step is the IB stage of every block then its fluid step."""

    def __init__(self, blocks):
        self.blocks = list(blocks)
        arr = (C.c_void_p * len(self.blocks))(*[b.h for b in self.blocks])
        h = C.c_void_p()
        _check(load_library().fsi_batch_create(C.byref(h), len(self.blocks), arr))
        self.h = h
        self.M = [b.Mtot for b in self.blocks]
        self.moff = np.concatenate([[0], np.cumsum(self.M)]).astype(int)

    def close(self):
        if getattr(self, "h", None):
            load_library().fsi_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ib_step(self, markers, vf=None, denIn=None, dt=None, Uref=None, ntol=3, dtol=1e-5, blktime=None):
        """markers: one (xyz, vel, area) per block (None for a block without
        bodies). Returns (list of eforce (M,3), iterations (n,), residual (n,))."""
        Mall = int(self.moff[-1])
        xyz = np.zeros(3 * max(Mall, 1))
        vel = np.zeros(3 * max(Mall, 1))
        area = np.zeros(max(Mall, 1))
        for c, mk in enumerate(markers):
            if self.M[c] == 0:
                continue
            m0, m1 = self.moff[c], self.moff[c + 1]
            xyz[3 * m0:3 * m1] = np.asarray(mk[0], dtype=np.float64).reshape(-1)
            vel[3 * m0:3 * m1] = np.asarray(mk[1], dtype=np.float64).reshape(-1)
            area[m0:m1] = np.asarray(mk[2], dtype=np.float64).reshape(-1)
        ef, its, res = self.ib_step_packed(xyz, vel, area, vf, denIn, dt, Uref, ntol, dtol, blktime)
        out = [ef[self.moff[c]:self.moff[c + 1]].copy() for c in range(len(self.blocks))]
        return out, its, res

    def ib_step_packed(self, xyz, vel, area, vf=None, denIn=None, dt=None, Uref=None, ntol=3, dtol=1e-5,
                       blktime=None, eforce=None):
        """the markers of all blocks packed in block order: xyz, vel (sum M, 3),
        area (sum M); returns (eforce (sum M, 3), iterations (n,), residual (n,))"""
        n = len(self.blocks)
        Mall = int(self.moff[-1])
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        if Mall and (xyz.size < 3 * Mall or vel.size < 3 * Mall or area.size < Mall):
            raise ValueError("packed marker arrays are shorter than the blocks' bodies")
        def per(v, default):
            a = np.full(n, default, dtype=np.float64) if v is None else np.asarray(v, dtype=np.float64)
            return np.ascontiguousarray(np.broadcast_to(a, (n,)))
        vfa = np.zeros(3 * n) if vf is None else np.ascontiguousarray(np.asarray(vf, dtype=np.float64).reshape(-1))
        den = per(denIn, 1.0)
        dta = np.ascontiguousarray(np.array([b.dh for b in self.blocks]) if dt is None else per(dt, 1.0))
        ur = per(Uref, 1.0)
        bt = per(blktime, 0.0)
        ef = np.empty(3 * max(Mall, 1)) if eforce is None else eforce
        its = np.zeros(n, dtype=np.int32)
        res = np.zeros(n)
        IPt = C.POINTER(C.c_int)
        _check(load_library().fsi_batch_ib_step(self.h, _dp(xyz), _dp(vel), _dp(area), _dp(vfa), _dp(den), _dp(dta),
                                                _dp(ur), int(ntol), dtol, _dp(bt), _dp(ef), its.ctypes.data_as(IPt),
                                                _dp(res)))
        return ef[:3 * Mall].reshape(-1, 3), its, res

    def tune(self, reps=10):
        """autotune the bulk kernel's CTA size; returns (threads, ms per step)"""
        t = C.c_int()
        ms = C.c_float()
        _check(load_library().fsi_batch_tune(self.h, int(reps), C.byref(t), C.byref(ms)))
        return t.value, ms.value

    def set_threads(self, threads):
        _check(load_library().fsi_batch_set_threads(self.h, int(threads)))


def continue_write(path, blocks, step, time):
    """write_continue_blocks (FluidDomain.f90:266-281): the continue file of
    the blocks' current fIn"""
    arr = (C.c_void_p * len(blocks))(*[b.h.value for b in blocks])
    _check(load_library().fsi_continue_write(os.fsencode(path), arr, len(blocks), int(step), float(time)))


def continue_read(path, blocks):
    """check_is_continue (FluidDomain.f90:127-236): re-grid the blocks' fIn
    from a continue file on the GPU; returns the file's (step, time)"""
    arr = (C.c_void_p * len(blocks))(*[b.h.value for b in blocks])
    step = C.c_int(0)
    t = C.c_double(0.0)
    _check(load_library().fsi_continue_read(os.fsencode(path), arr, len(blocks), C.byref(step), C.byref(t)))
    return step.value, t.value

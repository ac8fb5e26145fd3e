"""ctypes binding of the CPU FP64 oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module. It restates FSILBM3D's hot path on the CPU (see fsi_oracle.h
for the parity status) and is never part of the product path.
"""
import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build_oracle  # noqa: E402

Q = 19


class OrFlow(C.Structure):
    _fields_ = [
        ("denIn", C.c_double),
        ("uvwIn", C.c_double * 3),
        ("shearRateIn", C.c_double * 3),
        ("velocityKind", C.c_int),
        ("interpolateScheme", C.c_int),
        ("volumeForceIn", C.c_double * 3),
        ("volumeForceAmp", C.c_double),
        ("volumeForceFreq", C.c_double),
        ("volumeForcePhi", C.c_double),
        ("nu", C.c_double),
    ]


DP = C.POINTER(C.c_double)


class OrBlock(C.Structure):
    _fields_ = [
        ("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int),
        ("dh", C.c_double), ("xmin", C.c_double), ("ymin", C.c_double), ("zmin", C.c_double),
        ("xmax", C.c_double), ("ymax", C.c_double), ("zmax", C.c_double),
        ("bnd", C.c_int * 6),
        ("periodic", C.c_int * 3),
        ("model", C.c_int),
        ("tau", C.c_double), ("omega", C.c_double),
        ("mc", C.c_double * 361), ("mf", C.c_double * 361),
        ("volumeForce", C.c_double * 3),
        ("blktime", C.c_double),
        ("f", DP), ("u", DP), ("den", DP), ("force", DP), ("tau_all", DP),
        ("hw", DP * 6),
        ("hw_ready", C.c_int * 6),
        ("params", C.c_double * 10),
        ("omega2", C.c_double),
        ("nu", C.c_double),
    ]


class OrBody(C.Structure):
    _fields_ = [
        ("M", C.c_int),
        ("xyz", DP), ("vel", DP), ("area", DP), ("eforce", DP),
        ("ei", C.POINTER(C.c_int16)), ("ew", C.POINTER(C.c_float)),
    ]


class OrPair(C.Structure):
    _fields_ = [
        ("sds", C.c_int * 6), ("s", C.c_int * 6), ("f", C.c_int * 6),
        ("si", C.c_int * 6), ("fi", C.c_int * 6),
        ("xDimS", C.c_int), ("xDimF", C.c_int), ("yDimS", C.c_int),
        ("yDimF", C.c_int), ("zDimS", C.c_int), ("zDimF", C.c_int),
    ]


_lib = None
_kind = "parity"


def select_build(kind):
    """Choose the build this process loads ("parity", the default, or
    "timing": see build_oracle.py) before the first oracle call. Returns
    the build in use, which stays the loaded one once a call has been made."""
    global _kind
    if kind not in build_oracle.FLAGS:
        raise ValueError("unknown oracle build %r" % (kind,))
    if _lib is None:
        _kind = kind
    return _kind


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build(kind=_kind)
        L = C.CDLL(path)
        BP, FP, BDP = C.POINTER(OrBlock), C.POINTER(OrFlow), C.POINTER(OrBody)
        L.or_evaluate_velocity.argtypes = [FP, C.c_double, C.c_double, C.c_double, C.c_double, DP]
        L.or_feq_dist.argtypes = [C.c_double, DP, DP]
        L.or_mrt_matrices.argtypes = [C.c_double, DP, DP]
        L.or_block_setup.argtypes = [BP, FP]
        L.or_initialise_flow.argtypes = [BP, FP, C.c_double]
        L.or_init_tgv.argtypes = [BP, C.c_double, C.c_double]
        L.or_update_volume_force.argtypes = [BP, FP]
        for name in ("or_macro", "or_reset_force", "or_add_force", "or_collide", "or_halfway_set"):
            getattr(L, name).argtypes = [BP]
        L.or_stream.argtypes = [BP, DP]
        L.or_set_bc.argtypes = [BP, FP]
        L.or_set_bc.restype = C.c_int
        L.or_ib_stencil.argtypes = [BDP, BP]
        L.or_ib_stencil.restype = C.c_int
        L.or_ib_penalty.argtypes = [BDP, C.c_int, BP, C.c_double, C.c_double, C.c_double,
                                    C.c_int, C.c_double, C.POINTER(C.c_int), DP]
        L.or_ib_spread.argtypes = [BDP, C.c_int, BP]
        L.or_step.argtypes = [BP, FP, BDP, C.c_int, C.c_double, C.c_int, C.c_double, DP,
                              C.POINTER(C.c_int), DP]
        L.or_step.restype = C.c_int
        L.or_field_stat.argtypes = [BP, C.c_double, DP, DP]
        L.or_build_pair.argtypes = [BP, BP, C.POINTER(OrPair)]
        L.or_grid_transform.argtypes = [DP, C.c_double, DP, C.c_double]
        BUF = (DP * 2) * 6
        L.or_extract_layer.argtypes = [BP, BP, C.POINTER(OrPair), C.c_int, BUF, BUF]
        L.or_interp_f2s.argtypes = [BP, BP, C.POINTER(OrPair), C.c_int, BUF, BUF, C.c_int]
        L.or_deliver_s2f.argtypes = [BP, BP, C.POINTER(OrPair)]
        L.or_continue_order.argtypes = [C.c_int, DP, C.POINTER(C.c_int)]
        L.or_continue_regrid.argtypes = [BP, C.c_int, BP, C.POINTER(C.c_int)]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(DP)


def make_flow(denIn=1.0, uvwIn=(0.0, 0.0, 0.0), shearRateIn=(0.0, 0.0, 0.0), velocityKind=0,
              interpolateScheme=1, volumeForceIn=(0.0, 0.0, 0.0), volumeForceAmp=0.0,
              volumeForceFreq=0.0, volumeForcePhi=0.0, nu=0.01):
    fl = OrFlow()
    fl.denIn = denIn
    fl.uvwIn[:] = list(uvwIn)
    fl.shearRateIn[:] = list(shearRateIn)
    fl.velocityKind = velocityKind
    fl.interpolateScheme = interpolateScheme
    fl.volumeForceIn[:] = list(volumeForceIn)
    fl.volumeForceAmp = volumeForceAmp
    fl.volumeForceFreq = volumeForceFreq
    fl.volumeForcePhi = volumeForcePhi
    fl.nu = nu
    return fl


class Block:
    """One oracle block; numpy arrays in the reference's (z,y,x,q) order,
    exposed with shape (q, x, y, z) in C order (same memory)."""

    def __init__(self, X, Y, Z, dh, origin, bnd, model, flow, with_tau=True, params=None):
        self.b = OrBlock()
        b = self.b
        b.X, b.Y, b.Z = X, Y, Z
        b.dh = dh
        b.xmin, b.ymin, b.zmin = origin
        b.bnd[:] = list(bnd)
        b.model = model
        if params is not None:
            b.params[:len(params)] = list(params)
        n = X * Y * Z
        self.n = n
        self.f = np.zeros(Q * n)
        self.u = np.zeros(3 * n)
        self.den = np.zeros(n)
        self.force = np.zeros(3 * n)
        self.tau_all = np.zeros(n) if with_tau else None
        self.tmp = np.zeros(Q * n)
        b.f, b.u, b.den, b.force = _dp(self.f), _dp(self.u), _dp(self.den), _dp(self.force)
        b.tau_all = _dp(self.tau_all) if with_tau else DP()
        self.hw = []
        for k in range(6):
            ax = k // 2
            A, B = [(Z, Y), (Z, X), (Y, X)][ax]
            h = np.zeros(Q * A * B)
            self.hw.append(h)
            b.hw[k] = _dp(h)
        self.flow = flow
        lib().or_block_setup(C.byref(b), C.byref(flow))

    # views in (q, x, y, z) index order over the Fortran (z,y,x,q) memory
    def fview(self):
        return self.f.reshape(Q, self.b.X, self.b.Y, self.b.Z)

    def initialise(self, time=0.0):
        lib().or_initialise_flow(C.byref(self.b), C.byref(self.flow), time)

    def init_tgv(self, u0, rho0=1.0):
        lib().or_init_tgv(C.byref(self.b), u0, rho0)

    def set_bc(self):
        rc = lib().or_set_bc(C.byref(self.b), C.byref(self.flow))
        if rc != 0:
            raise RuntimeError("oracle: unknown boundary condition")

    def macro(self):
        lib().or_macro(C.byref(self.b))

    def collide(self):
        """collision_ alone on the current f, den, u and force"""
        lib().or_collide(C.byref(self.b))

    def step(self, bodies=(), Uref=1.0, ntol=0, dtol=0.0):
        arr = (OrBody * max(1, len(bodies)))()
        for i, bd in enumerate(bodies):
            arr[i] = bd.s
        it = C.c_int(0)
        res = C.c_double(0.0)
        rc = lib().or_step(C.byref(self.b), C.byref(self.flow), arr, len(bodies), Uref, ntol, dtol,
                           _dp(self.tmp), C.byref(it), C.byref(res))
        if rc != 0:
            raise RuntimeError("oracle step failed (%d)" % rc)
        return it.value, res.value

    def field_stat(self, Uref):
        l2 = np.zeros(3)
        li = np.zeros(3)
        lib().or_field_stat(C.byref(self.b), Uref, _dp(l2), _dp(li))
        return l2, li


class Body:
    def __init__(self, xyz, vel, area):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        self.vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1)
        self.area = np.ascontiguousarray(area, dtype=np.float64).reshape(-1)
        M = self.area.size
        self.eforce = np.zeros(3 * M)
        self.ei = np.zeros(12 * M, dtype=np.int16)
        self.ew = np.zeros(12 * M, dtype=np.float32)
        s = OrBody()
        s.M = M
        s.xyz, s.vel, s.area, s.eforce = _dp(self.xyz), _dp(self.vel), _dp(self.area), _dp(self.eforce)
        s.ei = self.ei.ctypes.data_as(C.POINTER(C.c_int16))
        s.ew = self.ew.ctypes.data_as(C.POINTER(C.c_float))
        self.s = s


class Pair:
    """A father/son pair with its extracted face layers (CommPair and the
    fIn_F*/tau_F* buffers, LBMBlockComm.f90:11-18, 213-264)."""

    def __init__(self, father, son, scheme=1):
        self.fa, self.so, self.scheme = father, son, scheme
        self.p = OrPair()
        lib().or_build_pair(C.byref(father.b), C.byref(son.b), C.byref(self.p))
        p = self.p
        # interpolate_fIn (LBMBlockComm.f90:808-956) reads outside its face
        # arrays on narrow faces (under 5 son nodes a side with scheme 2, or a
        # last odd son node past the father's face): refused, as the library does
        for k in range(6):
            if son.b.bnd[k] != 0:
                continue
            ax = k // 2
            AF, BF = [(p.zDimF, p.yDimF), (p.zDimF, p.xDimF), (p.yDimF, p.xDimF)][ax]
            AS, BS = [(p.zDimS, p.yDimS), (p.zDimS, p.xDimS), (p.yDimS, p.xDimS)][ax]
            AO, BO = (AS if AS % 2 else AS - 1), (BS if BS % 2 else BS - 1)
            ok = (AO + 1) // 2 <= AF and (BO + 1) // 2 <= BF and (scheme != 2 or min(AS, BS) >= 5)
            if not ok:
                raise ValueError("son face %d too narrow for interpolation scheme %d" % (k, scheme))
        self.keep = []
        self.bf = ((DP * 2) * 6)()
        self.bt = ((DP * 2) * 6)()
        for k in range(6):
            ax = k // 2
            A, B = [(p.zDimF, p.yDimF), (p.zDimF, p.xDimF), (p.yDimF, p.xDimF)][ax]
            for t in range(2):
                f = np.zeros(19 * A * B)
                tt = np.zeros(A * B)
                self.keep += [f, tt]
                self.bf[k][t] = _dp(f)
                self.bt[k][t] = _dp(tt)

    def extract(self, level):
        lib().or_extract_layer(C.byref(self.fa.b), C.byref(self.so.b), C.byref(self.p), level, self.bf, self.bt)

    def father_to_son(self, n_timeStep):
        lib().or_interp_f2s(C.byref(self.so.b), C.byref(self.fa.b), C.byref(self.p), n_timeStep, self.bf, self.bt,
                            self.scheme)

    def son_to_father(self):
        lib().or_deliver_s2f(C.byref(self.fa.b), C.byref(self.so.b), C.byref(self.p))


def block_stage_pre(b):
    """update_volume_force_ .. add_volume_force_ without bodies"""
    L = lib()
    L.or_update_volume_force(C.byref(b.b), C.byref(b.flow))
    L.or_macro(C.byref(b.b))
    L.or_reset_force(C.byref(b.b))
    L.or_add_force(C.byref(b.b))


def block_stage_post(b):
    """collision_ .. set_boundary_conditions_"""
    L = lib()
    L.or_collide(C.byref(b.b))
    L.or_halfway_set(C.byref(b.b))
    L.or_stream(C.byref(b.b), _dp(b.tmp))
    if L.or_set_bc(C.byref(b.b), C.byref(b.flow)) != 0:
        raise RuntimeError("oracle: unknown boundary condition")


def feq(density, vel):
    out = np.zeros(Q)
    v = np.asarray(vel, dtype=np.float64)
    lib().or_feq_dist(density, _dp(v), _dp(out))
    return out


def mrt_matrices(omega):
    mc = np.zeros(361)
    mf = np.zeros(361)
    lib().or_mrt_matrices(omega, _dp(mc), _dp(mf))
    return mc.reshape(19, 19, order="F"), mf.reshape(19, 19, order="F")


# ---------------------------------------------------------------- outputs
# Restatements of the reference's output arithmetic on den/uuu (FP64, the
# reference's operation order), for the checks of the packing kernels.

def pack_flow(den, u, X, Y, Z, off, denIn, Uref):
    """write_flow_, FluidDomain.f90:1651-1663: FP32 (4, nx, ny, nz) of
    p = Cs2 (den - denIn), u/Uref over the block minus `off` cells per side"""
    d = np.asarray(den).reshape(X, Y, Z)[off:X - off, off:Y - off, off:Z - off]
    uu = np.asarray(u).reshape(3, X, Y, Z)[:, off:X - off, off:Y - off, off:Z - off]
    inv = 1.0 / Uref
    out = np.empty((4,) + d.shape, dtype=np.float32)
    out[0] = ((1.0 / 3.0) * (d - denIn)).astype(np.float32)
    for k in range(3):
        out[1 + k] = (uu[k] * inv).astype(np.float32)
    return out


def flux(den, u, X, Y, Z, dh, denIn, Uref, Yref, Zref):
    """write_fluid_flux, FluidDomain.f90:2019-2056 (serial sums, z outer)"""
    d = np.asarray(den).reshape(X, Y, Z)
    ux = np.asarray(u).reshape(3, X, Y, Z)[0]
    res = []
    for x in (0, (X + 1) // 2 - 1, X - 1):
        s = 0.0
        for k in range(Z):
            wz = 0.5 if (k == 0 or k == Z - 1) else 1.0
            for j in range(Y):
                wy = 0.5 if (j == 0 or j == Y - 1) else 1.0
                s = s + ((((float(ux[x, j, k]) * float(d[x, j, k])) * dh) * dh) * wy) * wz
        res.append(s / (((denIn * Uref) * Zref) * Yref))
    return np.array(res)


def probe(u, X, Y, Z, dh, origin, point, Uref):
    """grid_value_interpolation, Util.f90:123-158, for the three components"""
    xmin, ymin, zmin = origin
    uu = np.asarray(u).reshape(3, X, Y, Z)
    cx, cy, cz = point
    x1 = int(np.floor((cx - xmin) / dh + 1.0)); y1 = int(np.floor((cy - ymin) / dh + 1.0))
    z1 = int(np.floor((cz - zmin) / dh + 1.0))
    x2, y2, z2 = min(x1 + 1, X), min(y1 + 1, Y), min(z1 + 1, Z)
    dx1 = cx - (xmin + dh * (x1 - 1)); dy1 = cy - (ymin + dh * (y1 - 1)); dz1 = cz - (zmin + dh * (z1 - 1))
    dx2, dy2, dz2 = dh - dx1, dh - dy1, dh - dz1
    co = 1.0 / ((dh * dh) * dh)
    c = [((dx2 * dy2) * dz2) * co, ((dx2 * dy2) * dz1) * co, ((dx2 * dy1) * dz2) * co, ((dx1 * dy2) * dz2) * co,
         ((dx2 * dy1) * dz1) * co, ((dx1 * dy2) * dz1) * co, ((dx1 * dy1) * dz2) * co, ((dx1 * dy1) * dz1) * co]
    idx = [(z1, y1, x1), (z2, y1, x1), (z1, y2, x1), (z1, y1, x2), (z2, y2, x1), (z2, y1, x2), (z1, y2, x2),
           (z2, y2, x2)]
    out = []
    for k in range(3):
        v = 0.0
        for ci, (z, y, x) in zip(c, idx):
            v = v + ci * float(uu[k, x - 1, y - 1, z - 1])
        out.append(v * (1.0 / Uref))
    return np.array(out)


# ---- continue files (write_continue_blocks / write_continue_ /
# read_continue_, FluidDomain.f90:266-281, 1770-1789): stream access, native
# byte order: int32 nblocks, int32 step, real8 time; per block real8 xmin,
# ymin, zmin, dh, int32 xDim, yDim, zDim, real8 fIn(z,y,x,0:18)

def write_continue(path, step, time, blocks):
    """blocks: (xmin, ymin, zmin, dh, f) with f of shape (19, X, Y, Z)"""
    with open(path, "wb") as fh:
        fh.write(np.array([len(blocks), step], dtype="<i4").tobytes())
        fh.write(np.array([time], dtype="<f8").tobytes())
        for xmin, ymin, zmin, dh, f in blocks:
            fh.write(np.array([xmin, ymin, zmin, dh], dtype="<f8").tobytes())
            fh.write(np.array(f.shape[1:], dtype="<i4").tobytes())
            fh.write(np.ascontiguousarray(f, dtype="<f8").tobytes())


def read_continue(path):
    """(step, time, [(xmin, ymin, zmin, dh, f (19, X, Y, Z))])"""
    raw = open(path, "rb").read()
    n, step = np.frombuffer(raw, "<i4", 2, 0)
    time = float(np.frombuffer(raw, "<f8", 1, 8)[0])
    off = 16
    out = []
    for _ in range(int(n)):
        xmin, ymin, zmin, dh = np.frombuffer(raw, "<f8", 4, off)
        X, Y, Z = (int(v) for v in np.frombuffer(raw, "<i4", 3, off + 32))
        off += 44
        f = np.frombuffer(raw, "<f8", 19 * X * Y * Z, off).reshape(19, X, Y, Z).copy()
        off += 8 * f.size
        out.append((float(xmin), float(ymin), float(zmin), float(dh), f))
    return int(step), time, out


def continue_regrid(block, olds):
    """check_is_continue's re-grid of block.f from olds = [(xmin, ymin, zmin,
    dh, f)] (cells outside every old block keep their values)"""
    keep = []
    arr = (OrBlock * max(1, len(olds)))()
    for k, (xmin, ymin, zmin, dh, f) in enumerate(olds):
        fc = np.ascontiguousarray(f, dtype=np.float64)
        keep.append(fc)
        o = arr[k]
        o.X, o.Y, o.Z = fc.shape[1:]
        o.dh, o.xmin, o.ymin, o.zmin = dh, xmin, ymin, zmin
        o.f = _dp(fc)
    dhs = np.array([o[3] for o in olds], dtype=np.float64)
    order = (C.c_int * max(1, len(olds)))()
    lib().or_continue_order(len(olds), _dp(dhs), order)
    lib().or_continue_regrid(C.byref(block.b), len(olds), arr, order)
    return list(order)[:len(olds)]

"""Host side of a flexible body: the plate's beam mesh file and the structural
solver of include/fsi_beam.h (host C++, FP64, no device work).

The reference reads a body's beam from its mesh file (``plate.dat``,
Beam_ReadBuild, SolidSolver.f90:1270-1399), places Nspan immersed-boundary
markers per beam element (PlateUpdatePosVelArea_, Solidbody.f90:604-646),
collects the Lagrangian force into the beam load (FluidVolumeForce_,
Solidbody.f90:946-967) and advances the beam once per fluid step
(Beam_structure, SolidSolver.f90:1820-1877). ``Plate`` holds one such body;
``read_plate_dat`` and ``write_plate_dat`` restate the file format, and
``plate_mesh`` builds the mesh of a rectangular plate whose beam runs along
the chord.
"""
import ctypes as C

import numpy as np

from .abi import FsiError, _check, load_library

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)


class BeamParams(C.Structure):
    """fsi_beam_params: Set_SolidSolver_Params (SolidSolver.f90:1249-1264)."""
    _fields_ = [("dampK", C.c_double), ("dampM", C.c_double), ("GeoGamma", C.c_double),
                ("NewmarkGamma", C.c_double), ("NewmarkBeta", C.c_double), ("dtolFEM", C.c_double),
                ("ntolFEM", C.c_int), ("isKB", C.c_int), ("g", C.c_double * 3)]


class BeamBody(C.Structure):
    """fsi_beam_body: Beam_SetSolver (SolidSolver.f90:1219-1248), angles and
    phases in degrees as inFlow.dat gives them."""
    _fields_ = [("iBodyModel", C.c_int), ("isMotionGiven", C.c_int * 6),
                ("denR", C.c_double), ("psR", C.c_double), ("EmR", C.c_double), ("tcR", C.c_double),
                ("KB", C.c_double), ("KS", C.c_double), ("Freq", C.c_double), ("St", C.c_double),
                ("XYZo", C.c_double * 3), ("initXYZVel", C.c_double * 3), ("XYZAmpl", C.c_double * 3),
                ("XYZPhi", C.c_double * 3), ("AoAo", C.c_double * 3), ("AoAAmpl", C.c_double * 3),
                ("AoAPhi", C.c_double * 3)]


def _declare(L):
    if getattr(L, "_beam_declared", False):
        return L
    VP = C.c_void_p
    L.fsi_beam_create.argtypes = [C.POINTER(VP), C.POINTER(BeamParams), C.POINTER(BeamBody), C.c_int, C.c_int,
                                  C.c_int, DP, DP, IP, IP, DP, DP]
    L.fsi_beam_destroy.argtypes = [VP]
    L.fsi_beam_set_material.argtypes = [VP, C.c_double, C.c_double, C.c_double, DP, DP, DP]
    L.fsi_beam_initialise.argtypes = [VP, C.c_double, IP]
    L.fsi_beam_markers.argtypes = [VP, C.c_double, C.c_double, DP, DP, DP]
    L.fsi_beam_load.argtypes = [VP, DP, DP]
    L.fsi_beam_structure.argtypes = [VP, C.c_double, C.c_int, C.c_double, C.c_double, IP, DP]
    L.fsi_beam_state.argtypes = [VP, DP, DP, DP, DP, DP]
    L.fsi_beam_info.argtypes = [VP, IP, IP, DP]
    L._beam_declared = True
    return L


def _dp(a):
    return a.ctypes.data_as(DP)


def _ip(a):
    return a.ctypes.data_as(IP)


def _sections(path):
    """The lines of a mesh file and the line index of each section name. The
    reference finds a section by list-directed reading of each line's first
    item and comparing it with the name (FindSection, SolidSolver.f90:1352-1369)."""
    lines = open(path).read().splitlines()
    heads = {}
    for i, ln in enumerate(lines):
        first = ln.replace(",", " ").split()
        if first and first[0] not in heads:
            heads[first[0]] = i
    return lines, heads


def _fnum(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def read_plate_dat(path):
    """Beam_ReadBuild's file (SolidSolver.f90:1270-1350): a title line, then
    nND nEL nMT; sections POINT (id, x, y, z, Lspan, Rspan, dirX, dirY, dirZ),
    MATERIAL (id, E, G, A, RHO, GAMMA, JT, IY, IZ), CONSTRAINT (id and six
    0/1 flags) and ELEMENT (id, i, j, k, TYPE, MAT, Nspan), each after a count
    that must match. Returns a dict of numpy arrays in the reference's
    column-major shapes, transposed: xyz (nND, 8), material (nMT, 8),
    boundary (nND, 6), elements (nEL, 6), ordered by id."""
    lines, heads = _sections(path)
    nND, nEL, nMT = (int(v) for v in lines[1].replace(",", " ").split()[:3])

    def rows(name, n, width):
        if name not in heads:
            raise FsiError(-1, "cannot find section %s in %s" % (name, path))
        i = heads[name] + 1
        count = int(lines[i].split()[0])
        if count != n:
            raise FsiError(-1, "%s number inconsistent (%d, %d expected)" % (name, count, n))
        out = []
        for ln in lines[i + 1:i + 1 + n]:
            tok = ln.replace(",", " ").split()
            out.append((int(tok[0]), tok[1:1 + width]))
        return out

    xyz = np.zeros((nND, 8))
    for k, (tid, v) in enumerate(rows("POINT", nND, 8)):
        xyz[k] = [_fnum(t) for t in v]
    material = np.zeros((nMT, 8))
    for k, (tid, v) in enumerate(rows("MATERIAL", nMT, 8)):
        material[k] = [_fnum(t) for t in v]
    boundary = np.zeros((nND, 6), dtype=np.int32)
    for k, (tid, v) in enumerate(rows("CONSTRAINT", nND, 6)):
        boundary[k] = [int(t) for t in v]
    elements = np.zeros((nEL, 6), dtype=np.int32)
    seen = np.zeros(nEL, dtype=bool)
    for tid, v in rows("ELEMENT", nEL, 6):
        if 1 <= tid <= nEL:
            elements[tid - 1] = [int(t) for t in v]
            seen[tid - 1] = True
    if not seen.all():
        raise FsiError(-1, "ELEMENT ids do not cover 1..%d" % nEL)
    return dict(nND=nND, nEL=nEL, nMT=nMT, xyz=xyz, material=material, boundary=boundary, elements=elements)


def write_plate_dat(path, mesh, title="Frame3D : point number, element number, material number"):
    """Write a mesh dict in the layout SurfacetoBeam_write produces
    (Solidbody.f90:1149-1168)."""
    with open(path, "w") as f:
        f.write(title + "\n")
        f.write("%5d%5d%5d\n" % (mesh["nND"], mesh["nEL"], mesh["nMT"]))
        f.write("POINT\n")
        f.write("%5d" % mesh["nND"] + "".join(" %20s" % n for n in
                                            ("X", "Y", "Z", "Lspan", "Rspan", "dirX", "dirY", "dirZ")) + "\n")
        for i, r in enumerate(mesh["xyz"]):
            f.write("%5d" % (i + 1) + "".join(" %20.10f" % v for v in r) + "\n")
        f.write("ELEMENT\n")
        f.write("%5d%6s%6s%6s%6s%6s%6s\n" % (mesh["nEL"], "I", "J", "K", "TYPE", "MAT", "Nspan"))
        for i, r in enumerate(mesh["elements"]):
            f.write("%5d" % (i + 1) + "".join("%6d" % v for v in r) + "\n")
        f.write("CONSTRAINT\n")
        f.write("%5d%6s%6s%6s%6s%6s%6s\n" % (mesh["nND"], "XTRA", "YTRA", "ZTRA", "XROT", "YROT", "ZROT"))
        for i, r in enumerate(mesh["boundary"]):
            f.write("%5d" % (i + 1) + "".join("%6d" % v for v in r) + "\n")
        f.write("MATERIAL\n")
        f.write("%5d%12s%12s%12s%12s%12s%12s%12s%12s\n" % (mesh["nMT"], "E", "G", "A", "RHO", "GAMMA", "JT", "IY",
                                                         "IZ"))
        for i, r in enumerate(mesh["material"]):
            f.write("%5d" % (i + 1) + "".join("%24.15E" % v for v in r) + "\n")
        f.write("END\n")


def plate_mesh(n_chord, chord=1.0, span=1.0, n_span=None, clamp_leading_edge=True,
               material=(1.0, 0.5, 1.0, 1.0, 0.0, 1.0, 1.0, 1.0)):
    """The beam mesh of a flat chord x span plate: n_chord elements along x
    from the body reference point (node 1 at the origin, the leading edge),
    each carrying n_span markers over the span (Lspan = Rspan = span/2, span
    direction +z); node 1 constrained (all six flags 1, which Beam_adjustBC
    turns into the body's prescribed DOFs) when clamp_leading_edge. The
    material row is overwritten from EmR/tcR or KB/KS when isKB is 0 or 1."""
    n_span = n_chord if n_span is None else n_span
    nND = n_chord + 1
    xyz = np.zeros((nND, 8))
    xyz[:, 0] = chord * np.arange(nND) / n_chord
    xyz[:, 3] = 0.5 * span
    xyz[:, 4] = 0.5 * span
    xyz[:, 7] = 1.0
    boundary = np.zeros((nND, 6), dtype=np.int32)
    if clamp_leading_edge:
        boundary[0] = 1
    elements = np.zeros((n_chord, 6), dtype=np.int32)
    for e in range(n_chord):
        elements[e] = (e + 1, e + 2, e + 2, 2, 1, n_span)
    return dict(nND=nND, nEL=n_chord, nMT=1, xyz=xyz, material=np.array([material], dtype=np.float64),
                boundary=boundary, elements=elements)


class Plate:
    """One plate body: its beam (BeamSolver) and its markers (VirtualBody of
    type 1). ``solver`` and ``body`` are keyword dicts of fsi_beam_params
    and fsi_beam_body; the material and the initial state follow the
    reference's set-up order (Beam_ReadBuild, Beam_calculate_angle_material,
    Beam_Initialise, PlateBuild_)."""

    def __init__(self, mesh, solver, body, Lref=1.0, Uref=1.0, denIn=1.0, uvwIn=(0.0, 0.0, 0.0), alpha=1.0,
                 time=0.0):
        L = _declare(load_library())
        self._L = L
        sp = BeamParams(**{k: v for k, v in solver.items() if k != "g"})
        sp.g[:] = list(solver.get("g", (0.0, 0.0, 0.0)))
        bp = BeamBody()
        for k, v in body.items():
            if isinstance(getattr(bp, k), C.Array):
                getattr(bp, k)[:] = list(v)
            else:
                setattr(bp, k, v)
        self.mesh = mesh
        xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64)
        mat = np.ascontiguousarray(mesh["material"], dtype=np.float64)
        bnd = np.ascontiguousarray(mesh["boundary"], dtype=np.int32)
        ele = np.ascontiguousarray(mesh["elements"], dtype=np.int32)
        h = C.c_void_p()
        asfac, lchod = C.c_double(), C.c_double()
        _check(L.fsi_beam_create(C.byref(h), C.byref(sp), C.byref(bp), mesh["nND"], mesh["nEL"], mesh["nMT"],
                                 _dp(xyz), _dp(mat), _ip(bnd), _ip(ele), C.byref(asfac), C.byref(lchod)))
        self.h = h
        self.Asfac, self.Lchod = asfac.value, lchod.value
        self.nND, self.nEL = mesh["nND"], mesh["nEL"]
        umax, lthck = C.c_double(0.0), C.c_double()
        uin = np.array(uvwIn, dtype=np.float64)
        _check(L.fsi_beam_set_material(h, Lref, Uref, denIn, _dp(uin), C.byref(umax), C.byref(lthck)))
        self.uMax, self.Lthck = umax.value, lthck.value
        m = C.c_int()
        _check(L.fsi_beam_initialise(h, time, C.byref(m)))
        self.M = m.value
        self.alpha, self.denIn, self.Lref = alpha, denIn, Lref
        self.XYZo = np.array(body.get("XYZo", (0.0, 0.0, 0.0)), dtype=np.float64)
        self.last_iters, self.last_dnorm = 0, 0.0

    def close(self):
        if getattr(self, "h", None):
            self._L.fsi_beam_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def markers(self):
        """PlateUpdatePosVelArea_: (xyz (M,3), vel (M,3), area (M,))"""
        xyz, vel, area = np.zeros((self.M, 3)), np.zeros((self.M, 3)), np.zeros(self.M)
        _check(self._L.fsi_beam_markers(self.h, self.alpha, self.denIn, _dp(xyz), _dp(vel), _dp(area)))
        return xyz, vel, area

    def load(self, xyz, eforce):
        """the beam load lodFlow from the markers' Lagrangian force"""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        ef = np.ascontiguousarray(eforce, dtype=np.float64)
        _check(self._L.fsi_beam_load(self.h, _dp(xyz), _dp(ef)))

    def structure(self, time, isubstep=1, deltat=1.0, subdeltat=None):
        """Beam_structure for sub-step isubstep of the fluid step ending at time"""
        it, dn = C.c_int(), C.c_double()
        sub = deltat if subdeltat is None else subdeltat
        _check(self._L.fsi_beam_structure(self.h, time, int(isubstep), deltat, sub, C.byref(it), C.byref(dn)))
        self.last_iters, self.last_dnorm = it.value, dn.value
        return it.value, dn.value

    def state(self):
        """node pos, dsp, vel, acc (nND, 6) and lodFlow (nND, 6)"""
        a = [np.zeros((self.nND, 6)) for _ in range(5)]
        _check(self._L.fsi_beam_state(self.h, *[_dp(v) for v in a]))
        return dict(zip(("pos", "dsp", "vel", "acc", "lodFlow"), a))

    def reference_point(self):
        xyz = np.zeros(3)
        _check(self._L.fsi_beam_info(self.h, None, None, _dp(xyz)))
        return xyz

    def tip(self):
        """the last node's position relative to the body origin over Lref, as
        Beam_write_solid_info writes it (SolidSolver.f90:1744-1745)"""
        pos = self.state()["pos"]
        return (pos[-1, :3] - self.XYZo) / self.Lref

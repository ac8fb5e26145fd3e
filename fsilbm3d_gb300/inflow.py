"""The fluid sections of the reference's input file inFlow.dat, read as the
reference reads them, and the block descriptors they give.

Restated behaviour (file:line of the reference):
  * a section starts at the first line whose first list-directed item
    contains the section keyword (found_keyword, Util.f90:55-75; the search
    restarts from the top for each section). The match is the reference's
    exactly: to_lowercase (Util.f90:78-87) declares its argument with length
    1, so only the first character of the keyword and of the item is folded
    to lower case; and INDEX searches for the keyword with its blank padding
    to 40 characters inside the item padded to 50, so the item must end with
    the keyword ('FlowCondition' and '#flowCondition' match;
    'flowcondition', 'FlowConditions' and '#FlowCondition' do not);
  * data lines are the next lines whose first non-blank character is not
    '#' (readNextData, Util.f90:89-104); a blank data line is an error, as
    the reference's list-directed read of it fails;
  * entries of a multi-entry section are separated by a line whose first
    item starts with '=' (readequal, Util.f90:106-121);
  * each data line is a Fortran list-directed read (items separated by
    blanks or commas, ``r*c`` repeats, ``r*`` null values, '/' ends the
    record, D exponents); items beyond those a read asks for are ignored.
Sections: Parallel and FlowCondition (read_flow_conditions,
FlowCondition.f90:31-77), the global lines of SolidBody (read_solid_files,
Solidbody.f90:100-115: penalty and structural-solver globals, the number of
bodies and groups; the bodies' own entries and mesh files are not read),
FluidBlocks (read_fuild_blocks, FluidDomain.f90:61-108, with
check_periodic_boundary_ :110-126), ProbingFluid and ProbingSolid
(read_probe_params, FlowCondition.f90:79-113). The reference scales of
calculate_reference_params (Solidbody.f90:219-284) are computed for the
choices that need no body data (or only the chord, when given).

Like the reference, a malformed file stops the run: here with
InFlowError.
"""
import math
import re
from dataclasses import dataclass, field
from typing import List, Optional

# ConstParams.f90:31-34
BC_PERIODIC = 301


class InFlowError(ValueError):
    pass


def _items(line):
    """The values of a list-directed record: strings, or None for a null
    value (``r*`` repeats and empty items between commas)."""
    out = []
    s = line
    cut = s.find("/")
    if cut >= 0:
        s = s[:cut]
    # separators: blanks, or one comma with optional blanks around it
    toks = re.split(r"\s*,\s*|\s+", s.strip())
    if toks == [""]:
        return out
    for t in toks:
        m = re.fullmatch(r"(\d+)\*(.*)", t)
        if m:
            r = int(m.group(1))
            out.extend([m.group(2) if m.group(2) != "" else None] * r)
        else:
            out.append(t if t != "" else None)
    return out


def _real(t):
    return float(t.replace("d", "e").replace("D", "e"))


def _int(t):
    return int(t)


def _read(line, kinds, what):
    """list-directed read of len(kinds) values ('i' or 'r') from one record;
    a null item leaves the value None (the variable keeps its old value in
    the reference)"""
    items = _items(line)
    if len(items) < len(kinds):
        raise InFlowError("%s: %d values expected in %r" % (what, len(kinds), line.rstrip("\n")))
    vals = []
    for k, t in zip(kinds, items):
        if t is None:
            vals.append(None)
            continue
        try:
            vals.append(_int(t) if k == "i" else _real(t))
        except ValueError:
            raise InFlowError("%s: cannot read %r in %r" % (what, t, line.rstrip("\n"))) from None
    return vals


class _Reader:
    def __init__(self, lines):
        self.lines = lines
        self.pos = 0

    def find(self, keyword):
        """found_keyword: from the top, the first record whose first item
        (character(50), first character folded to lower case) contains the
        keyword (character(40), first character folded, blank-padded)"""
        key = (keyword[:1].lower() + keyword[1:])[:40].ljust(40)
        word = "null"  # readString's initial value, kept through null items
        for i, line in enumerate(self.lines):
            items = _items(line)
            if not items:
                continue  # a list-directed read passes over blank records
            if items[0] is not None:
                word = items[0][:50]
            first = (word[:1].lower() + word[1:]).ljust(50)
            if key in first:
                self.pos = i + 1
                return
        raise InFlowError("%s is not found in inFlow.dat" % keyword)

    def next_data(self):
        """readNextData: the next record (character(256)) not starting with
        '#' after its leading blanks"""
        while self.pos < len(self.lines):
            line = self.lines[self.pos][:256]
            self.pos += 1
            if not line.lstrip().startswith("#"):
                return line
        raise InFlowError("end of file encounter in readNextData")

    def skip_to_equal(self):
        """readequal: past the next record whose first item starts with '='"""
        while self.pos < len(self.lines):
            items = _items(self.lines[self.pos])
            self.pos += 1
            if items and (items[0] or "").startswith("="):
                return
        raise InFlowError("end of file encounter in readequal")


@dataclass
class FlowConditions:
    """FlowCondType's inputs (FlowCondition.f90:11-26)"""
    npsize: int = 1
    isConCmpt: int = 0
    numsubstep: int = 1
    timeSimTotal: float = 0.0
    timeContiDelta: float = 0.0
    timeWriteBegin: float = 0.0
    timeWriteEnd: float = 0.0
    timeFlowDelta: float = 0.0
    timeBodyDelta: float = 0.0
    timeInfoDelta: float = 0.0
    Re: float = 0.0
    denIn: float = 1.0
    uvwIn: tuple = (0.0, 0.0, 0.0)
    shearRateIn: tuple = (0.0, 0.0, 0.0)
    velocityKind: int = 0
    volumeForceIn: tuple = (0.0, 0.0, 0.0)
    volumeForceAmp: float = 0.0
    volumeForceFreq: float = 0.0
    volumeForcePhi: float = 0.0
    LrefType: int = 0
    Lref: float = 0.0
    TrefType: int = 0
    Tref: float = 0.0
    UrefType: int = 0
    Uref: float = 0.0
    ntolLBM: int = 0
    dtolLBM: float = 0.0
    interpolateScheme: int = 1
    fluidProbingNum: int = 0
    inWhichBlock: int = 0
    fluidProbingCoords: List[tuple] = field(default_factory=list)
    solidProbingNum: int = 0
    solidProbingNode: List[int] = field(default_factory=list)
    # calculate_reference_params
    nu: Optional[float] = None


@dataclass
class SolidGlobals:
    """the global lines of the SolidBody section (Solidbody.f90:100-115)"""
    IBPenaltyAlpha: float = 1.0
    GeoGamma: float = 0.0
    NewmarkGamma: float = 0.0
    NewmarkBeta: float = 0.0
    dampK: float = 0.0
    dampM: float = 0.0
    dtolFEM: float = 0.0
    ntolFEM: int = 0
    nFish: int = 0
    nGroup: int = 0
    isKB: int = 0


@dataclass
class FluidBlock:
    """one entry of the FluidBlocks section (FluidDomain.f90:75-84)"""
    ID: int
    iCollidModel: int
    offsetOutput: int
    outputtype: int
    xDim: int
    yDim: int
    zDim: int
    dh: float
    xmin: float
    ymin: float
    zmin: float
    BndConds: tuple
    params: tuple
    periodic_bc: tuple = (0, 0, 0)
    xmax: float = 0.0
    ymax: float = 0.0
    zmax: float = 0.0


def _flow(r, fc):
    r.find("Parallel")
    (fc.npsize,) = _read(r.next_data(), "i", "Parallel")
    r.find("FlowCondition")
    fc.isConCmpt, fc.numsubstep = _read(r.next_data(), "ii", "isConCmpt, numsubstep")
    fc.timeSimTotal, fc.timeContiDelta = _read(r.next_data(), "rr", "timeSimTotal, timeContiDelta")
    fc.timeWriteBegin, fc.timeWriteEnd = _read(r.next_data(), "rr", "timeWriteBegin, timeWriteEnd")
    fc.timeFlowDelta, fc.timeBodyDelta, fc.timeInfoDelta = _read(r.next_data(), "rrr", "time deltas")
    fc.Re, fc.denIn = _read(r.next_data(), "rr", "Re, denIn")
    fc.uvwIn = tuple(_read(r.next_data(), "rrr", "uvwIn"))
    v = _read(r.next_data(), "rrri", "shearRateIn, velocityKind")
    fc.shearRateIn, fc.velocityKind = tuple(v[:3]), v[3]
    fc.volumeForceIn = tuple(_read(r.next_data(), "rrr", "volumeForceIn"))
    fc.volumeForceAmp, fc.volumeForceFreq, fc.volumeForcePhi = _read(r.next_data(), "rrr", "volume force wave")
    fc.LrefType, fc.Lref = _read(r.next_data(), "ir", "LrefType, Lref")
    fc.TrefType, fc.Tref = _read(r.next_data(), "ir", "TrefType, Tref")
    fc.UrefType, fc.Uref = _read(r.next_data(), "ir", "UrefType, Uref")
    fc.ntolLBM, fc.dtolLBM = _read(r.next_data(), "ir", "ntolLBM, dtolLBM")
    (fc.interpolateScheme,) = _read(r.next_data(), "i", "interpolateScheme")


def _solid(r):
    r.find("SolidBody")
    sg = SolidGlobals()
    sg.IBPenaltyAlpha, sg.GeoGamma = _read(r.next_data(), "rr", "IBPenaltyAlpha, GeoGamma")
    sg.NewmarkGamma, sg.NewmarkBeta = _read(r.next_data(), "rr", "NewmarkGamma, NewmarkBeta")
    sg.dampK, sg.dampM = _read(r.next_data(), "rr", "dampK, dampM")
    sg.dtolFEM, sg.ntolFEM = _read(r.next_data(), "ri", "dtolFEM, ntolFEM")
    sg.nFish, sg.nGroup, sg.isKB = _read(r.next_data(), "iii", "nFish, nGroup, isKB")
    if not sg.IBPenaltyAlpha > 1e-6:
        raise InFlowError("ERROR: IBPenaltyalpha should be positive (default 1) %g" % sg.IBPenaltyAlpha)
    return sg


def _blocks(r):
    r.find("FluidBlocks")
    (n,) = _read(r.next_data(), "i", "number of blocks")
    out = []
    for ib in range(n):
        ID, model, off, otype = _read(r.next_data(), "iiii", "ID, iCollidModel, offsetOutput, outputtype")
        X, Y, Z = _read(r.next_data(), "iii", "xDim, yDim, zDim")
        dh, xmin, ymin, zmin = _read(r.next_data(), "rrrr", "dh, xmin, ymin, zmin")
        bc = tuple(_read(r.next_data(), "iiiiii", "BndConds"))
        params = tuple(0.0 if p is None else p for p in _read(r.next_data(), "r" * 10, "params"))
        if ib < n - 1:
            r.skip_to_equal()
        if max(X, Y, Z) > 32767:
            raise InFlowError("Grid number exceeds 32767, please try to reduced the grid size.")
        periodic = []
        for i in range(3):
            lo, hi = bc[2 * i], bc[2 * i + 1]
            if lo == BC_PERIODIC or hi == BC_PERIODIC:
                if lo != hi:
                    raise InFlowError("Stop! Periodic boundaries must apper in pairs: %d %d" % (lo, hi))
                periodic.append(1)
            else:
                periodic.append(0)
        b = FluidBlock(ID, model, off, otype, X, Y, Z, dh, xmin, ymin, zmin, bc, params, tuple(periodic))
        b.xmax = xmin + dh * (X - 1) + (dh if periodic[0] else 0.0)
        b.ymax = ymin + dh * (Y - 1) + (dh if periodic[1] else 0.0)
        b.zmax = zmin + dh * (Z - 1) + (dh if periodic[2] else 0.0)
        out.append(b)
    return out


def _probes(r, fc):
    r.find("ProbingFluid")
    fc.fluidProbingNum, fc.inWhichBlock = _read(r.next_data(), "ii", "fluidProbingNum, inWhichBlock")
    fc.fluidProbingCoords = [tuple(_read(r.next_data(), "rrr", "probe")) for _ in range(max(0, fc.fluidProbingNum))]
    r.find("ProbingSolid")
    (fc.solidProbingNum,) = _read(r.next_data(), "i", "solidProbingNum")
    fc.solidProbingNode = [_read(r.next_data(), "i", "solid probe")[0] for _ in range(max(0, fc.solidProbingNum))]


def reference_scales(fc, nbodies=0, lchod=None):
    """calculate_reference_params (Solidbody.f90:219-284) for the choices
    that need no body data: Lref (type 0: 1 without bodies, the chord Lchod
    with bodies, which the caller passes), Uref (types 0-4, or the input
    value for types above 7), Tref (type 0 or the input), then
    nu = Uref Lref / Re. Choices that read the bodies' motion raise."""
    if fc.LrefType == 0:
        if nbodies:
            if lchod is None:
                raise InFlowError("LrefType 0 with bodies takes the chord Lchod of the solid input: pass lchod")
            fc.Lref = float(lchod)
        else:
            fc.Lref = 1.0
    u = fc.uvwIn
    if fc.UrefType == 0:
        fc.Uref = abs(u[0])
    elif fc.UrefType == 1:
        fc.Uref = abs(u[1])
    elif fc.UrefType == 2:
        fc.Uref = abs(u[2])
    elif fc.UrefType == 3:
        fc.Uref = math.sqrt(u[0] ** 2 + u[1] ** 2 + u[2] ** 2)
    elif fc.UrefType == 4:
        if fc.velocityKind != 2:
            raise InFlowError("oscillatory flow must set velocityKind to 2")
        fc.Uref = abs(fc.shearRateIn[0])
    elif fc.UrefType in (5, 6, 7):
        raise InFlowError("UrefType %d takes the bodies' frequencies and amplitudes" % fc.UrefType)
    if fc.TrefType == 0:
        fc.Tref = fc.Lref / fc.Uref
    elif fc.TrefType == 1:
        raise InFlowError("TrefType 1 takes the bodies' frequencies")
    fc.nu = fc.Uref * fc.Lref / fc.Re
    return fc


@dataclass
class InFlow:
    flow: FlowConditions
    blocks: List[FluidBlock]
    solid: SolidGlobals

    def block_kwargs(self, i, precision=None):
        """keyword arguments of fsilbm3d_gb300.Block for block i (an index
        into `blocks`), as initialise_ (FluidDomain.f90:433-545) sets the
        block up from the flow conditions"""
        if self.flow.nu is None:
            raise InFlowError("reference scales not computed (reference_scales)")
        b = self.blocks[i]
        kw = dict(xDim=b.xDim, yDim=b.yDim, zDim=b.zDim, dh=b.dh, origin=(b.xmin, b.ymin, b.zmin),
                  bndConds=b.BndConds, iCollidModel=b.iCollidModel, nu=self.flow.nu, denIn=self.flow.denIn,
                  uvwIn=self.flow.uvwIn, shearRateIn=self.flow.shearRateIn, velocityKind=self.flow.velocityKind,
                  params=b.params)
        if precision is not None:
            kw["precision"] = precision
        return kw


def read_inflow(path, probes=True, scales=True, lchod=None):
    """The fluid sections of inFlow.dat at `path` in the reference's order
    (main.f90:29-32): flow conditions, the SolidBody globals, blocks (and
    probes); with scales, the reference scales and nu (lchod: the bodies'
    chord, for LrefType 0 with bodies)."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    r = _Reader(lines)
    fc = FlowConditions()
    _flow(r, fc)
    solid = _solid(r)
    blocks = _blocks(r)
    if probes:
        _probes(r, fc)
    if scales:
        reference_scales(fc, nbodies=solid.nFish, lchod=lchod)
    return InFlow(fc, blocks, solid)

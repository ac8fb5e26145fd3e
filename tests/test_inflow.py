"""The inFlow.dat reader (fsilbm3d_gb300/inflow.py) against the reference's
reading rules, on synthetic files (runs without a GPU)."""
import inspect

import pytest

from fsilbm3d_gb300 import inflow as I

CASE = """\
# synthetic case: two blocks, one probe
Parallel
  8
FlowCondition
# isConCmpt numsubstep
0 2
40.0, 0.5
0.0 40.0
0.25 0.1 0.05
200.0 1.0d0
0.05 0.0 0.0
0.0 0.0 0.0 0
2*0.0 1.5D-6
0.0 0.0 0.0
0 1.0
0 1.0
0 0.05
5 1.0e-4
2
FluidBlocks
2
1 3 1 0
64 48 32
0.0625 -1.0 0.0 0.0
101 104 301 301 201 202
10*0.0
==========
2 2 0 0
32 24 16
0.03125 0.5 0.75 0.5
0 0 0 0 0 0
0.1875 9*0.0 / ignored tail
SolidBody
1.0 0.5
0.5 0.25
0.0 0.0
1.0e-6 20
0 0 1
ProbingFluid
2 1
0.5 1.5 1.0
1.0, 1.5, 0.5
ProbingSolid
1
7
"""


def write(tmp_path, text):
    p = tmp_path / "inFlow.dat"
    p.write_text(text)
    return str(p)


def test_reads_flow_blocks_and_probes(tmp_path):
    inf = I.read_inflow(write(tmp_path, CASE))
    fc = inf.flow
    assert fc.npsize == 8 and (fc.isConCmpt, fc.numsubstep) == (0, 2)
    assert (fc.timeSimTotal, fc.timeContiDelta) == (40.0, 0.5)
    assert (fc.Re, fc.denIn) == (200.0, 1.0) and fc.uvwIn == (0.05, 0.0, 0.0)
    assert fc.volumeForceIn == (0.0, 0.0, 1.5e-6)
    assert (fc.UrefType, fc.ntolLBM, fc.dtolLBM, fc.interpolateScheme) == (0, 5, 1e-4, 2)
    assert inf.solid.IBPenaltyAlpha == 1.0 and (inf.solid.nFish, inf.solid.nGroup, inf.solid.isKB) == (0, 0, 1)
    assert (inf.solid.dtolFEM, inf.solid.ntolFEM) == (1e-6, 20)
    assert fc.fluidProbingNum == 2 and fc.inWhichBlock == 1
    assert fc.fluidProbingCoords == [(0.5, 1.5, 1.0), (1.0, 1.5, 0.5)]
    assert fc.solidProbingNum == 1 and fc.solidProbingNode == [7]
    b0, b1 = inf.blocks
    assert (b0.ID, b0.iCollidModel, b0.offsetOutput) == (1, 3, 1)
    assert (b0.xDim, b0.yDim, b0.zDim, b0.dh) == (64, 48, 32, 0.0625)
    assert b0.BndConds == (101, 104, 301, 301, 201, 202) and b0.periodic_bc == (0, 1, 0)
    # xmax = xmin + dh (xDim - 1), one more dh on a periodic axis
    assert b0.xmax == -1.0 + 0.0625 * 63 and b0.ymax == 0.0625 * 48 and b0.zmax == 0.0625 * 31
    assert b1.ID == 2 and b1.params == (0.1875,) + (0.0,) * 9 and b1.BndConds == (0,) * 6
    # reference scales without bodies: Lref 1, Uref |u|, Tref Lref/Uref, nu
    assert fc.Lref == 1.0 and fc.Uref == 0.05 and fc.Tref == 1.0 / 0.05
    assert fc.nu == 0.05 * 1.0 / 200.0


def test_block_arguments_bind_to_the_block_constructor(tmp_path):
    import fsilbm3d_gb300 as F
    inf = I.read_inflow(write(tmp_path, CASE))
    kw = inf.block_kwargs(1, precision=F.PREC_F16)
    inspect.signature(F.Block).bind(**kw)
    assert kw["nu"] == inf.flow.nu and kw["origin"] == (0.5, 0.75, 0.5) and kw["iCollidModel"] == 2
    assert kw["params"][0] == 0.1875 and kw["uvwIn"] == (0.05, 0.0, 0.0)


@pytest.mark.parametrize("header,found", [
    ("FlowCondition", True), ("#flowCondition", True), ("  FlowCondition  extra words", True),
    ("flowcondition", False), ("FlowConditions", False), ("#FlowCondition", False),
])
def test_keyword_match_is_the_references(tmp_path, header, found):
    # only the first character is folded to lower case, and the blank-padded
    # keyword must end the line's first item
    text = CASE.replace("FlowCondition\n# isConCmpt", header + "\n# isConCmpt", 1)
    if found:
        assert I.read_inflow(write(tmp_path, text)).flow.numsubstep == 2
    else:
        with pytest.raises(I.InFlowError):
            I.read_inflow(write(tmp_path, text))


@pytest.mark.parametrize("edit,msg", [
    (("Parallel\n", "Paralel\n"), "Parallel is not found"),
    (("0 2\n", "0 2\n\n"), "values expected"),                  # a blank data line
    (("101 104 301 301 201 202", "101 104 301 101 201 202"), "pairs"),
    (("64 48 32", "64 48 40000"), "32767"),
    (("0 0.05\n5 1.0e-4", "5 0.05\n5 1.0e-4"), "UrefType 5"),
    (("==========\n", "----------\n"), "readequal"),
    (("1 3 1 0", "1 3.5 1 0"), "cannot read"),
    (("1.0 0.5\n0.5 0.25", "0.0 0.5\n0.5 0.25"), "IBPenaltyalpha"),
    (("0 0 1\n", "2 1 1\n"), "pass lchod"),                 # bodies, LrefType 0, no chord given
])
def test_malformed_files_stop(tmp_path, edit, msg):
    with pytest.raises(I.InFlowError, match=msg):
        I.read_inflow(write(tmp_path, CASE.replace(*edit, 1)))


def test_list_directed_items():
    assert I._items("1, 2  3*0.5 , 2* / tail 9") == ["1", "2", "0.5", "0.5", "0.5", None, None]
    assert I._items("   ") == [] and I._items("a,,b") == ["a", None, "b"]
    assert I._read("1.d0 2.5D-3 7", "rri", "x") == [1.0, 2.5e-3, 7]


def test_chord_sets_the_reference_length_with_bodies(tmp_path):
    inf = I.read_inflow(write(tmp_path, CASE.replace("0 0 1\n", "2 1 1\n", 1)), lchod=2.0)
    assert inf.solid.nFish == 2 and inf.flow.Lref == 2.0 and inf.flow.nu == 0.05 * 2.0 / 200.0

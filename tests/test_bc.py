"""Host-side boundary-condition tables: the mirror of the reference's
BC::Operator::Elastic::Constant / TensionTest and of the time interpolator
Numeric::Interpolator::Linear that their values are (no GPU)."""
import numpy as np
import pytest

from alamo_gb300 import bc as B


def test_interpolator_constant_and_ramp():
    assert B.Linear(0.25)(-3.0) == 0.25 and B.Linear("0.25")(7.0) == 0.25
    ramp = B.Linear("(0,1:0,0.01)")
    assert ramp(-1.0) == 0.0
    assert ramp(0.0) == 0.0
    assert ramp(0.5) == pytest.approx(0.005, rel=0, abs=1e-18)
    assert ramp(1.0) == 0.01
    assert ramp(2.0) == 0.01


def test_interpolator_piecewise():
    # the example of src/Numeric/Interpolator/Linear.H:27-35 (':' separates
    # times from values in the parser, Linear.H:82-87)
    f = B.Linear("(1.0,1.5,2.0:0.0,0.1,0.0)")
    assert f(0.5) == 0.0
    assert f(1.25) == pytest.approx(0.05)
    assert f(1.5) == pytest.approx(0.1)
    assert f(1.75) == pytest.approx(0.05)
    assert f(3.0) == 0.0


def test_interpolator_uniform_search_start():
    """Linear.H:135-141 starts the search at the interval a uniform spacing
    predicts; with non-uniform times it can start past the right interval and
    then returns the last value.  The mirror keeps that behaviour."""
    f = B.Linear("(0,1,10,11:0,1,2,3)")
    assert f(0.5) == pytest.approx(0.5)
    assert f(10.5) == pytest.approx(2.5)
    assert f(5.0) == 3.0  # the interval [1, 10] is skipped: start = 5 - 1 -> 2
    g = B.Linear("(0,1,10:0,1,2)")
    assert g(5.0) == pytest.approx(1 + 4 / 9)  # the clamp to n - 2 keeps [1, 10]


@pytest.mark.parametrize("bad", ["(0,1:0", "0,1:0,1)", "(0,1;0,1)", "(0,1:0)", "(1,0:0,1)"])
def test_interpolator_rejects_malformed(bad):
    with pytest.raises(ValueError):
        B.Linear(bad)


def test_constant_defaults_and_parse_with_time():
    bc = B.Constant()
    bt, bv = bc.tables()
    assert bt.shape == (26, 3) and bt.dtype == np.int32 and np.all(bt == B.DISPLACEMENT)
    assert bv.shape == (26, 3) and np.all(bv == 0.0)
    bc = B.Constant.parse({"type.xhi": "disp trac neumann", "val.xhi": "(0,2:0,1) 0.5 -1",
                           "type.zloxhi": "traction displacement periodic"})
    bt, bv = bc.tables(1.0)
    f = B.FACE["xhi"]
    assert list(bt[f]) == [B.DISPLACEMENT, B.TRACTION, B.NEUMANN]
    assert list(bv[f]) == [0.5, 0.5, -1.0]
    assert list(bt[B.FACE["zloxhi"]]) == [B.TRACTION, B.DISPLACEMENT, B.PERIODIC]
    assert bc.tables(4.0)[1][f, 0] == 1.0
    assert bc.tables(0.0)[1][f, 0] == 0.0
    bc.set("xhi", 0, "disp", 0.3)  # a constant replaces the interpolator
    assert bc.tables(1.0)[1][f, 0] == 0.3
    with pytest.raises(KeyError):
        B.Constant.parse({"typo.xhi": "disp disp disp"})


def _regions(tbl, comp, kind):
    return {B.FACES[f] for f in range(26) if tbl[f, comp] == kind}


XHI = {"xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi"}
XLO = {"xlo", "xloylo", "xloyhi", "zloxlo", "zhixlo", "xloylozlo", "xloylozhi", "xloyhizlo", "xloyhizhi"}
YLO = {"ylo", "xloylo", "xhiylo", "ylozlo", "ylozhi", "xloylozlo", "xloylozhi", "xhiylozlo", "xhiylozhi"}
YHI = {"yhi", "xloyhi", "xhiyhi", "yhizlo", "yhizhi", "xloyhizlo", "xloyhizhi", "xhiyhizlo", "xhiyhizhi"}
ZLO = {"zlo", "ylozlo", "yhizlo", "zloxlo", "zloxhi", "xloylozlo", "xloyhizlo", "xhiylozlo", "xhiyhizlo"}
ZHI = {"zhi", "ylozhi", "yhizhi", "zhixlo", "zhixhi", "xloylozhi", "xloyhizhi", "xhiylozhi", "xhiyhizhi"}


def test_tension_clamp():
    """uniaxial_stress_clamp (TensionTest.H:72-101): x-hi face, edges and
    corners pull u_x; y/z faces and yz edges traction-free; the rest fixed."""
    bt, bv = B.TensionTest("uniaxial_stress_clamp", disp="(0,1:0,0.1)").tables(0.5)
    free = {"ylo", "yhi", "zlo", "zhi", "ylozlo", "yhizlo", "ylozhi", "yhizhi"}
    for c in range(3):
        assert _regions(bt, c, B.TRACTION) == free
        assert _regions(bt, c, B.DISPLACEMENT) == set(B.FACES) - free
    assert {B.FACES[f] for f in range(26) if bv[f, 0] != 0} == XHI
    assert np.allclose(bv[[B.FACE[f] for f in XHI], 0], 0.05)
    assert np.all(bv[:, 1:] == 0)


def test_tension_kolsky():
    bt, bv = B.TensionTest("uniaxial_kolsky", disp=0.2).tables()
    for c in range(3):
        assert _regions(bt, c, B.TRACTION) == {"ylo", "yhi"}
    assert {B.FACES[f] for f in range(26) if bv[f, 0] != 0} == {"xlo", "xloylo", "xloyhi"}


@pytest.mark.parametrize("mode", ["disp", "trac"])
def test_tension_uniaxial_stress(mode):
    """uniaxial_stress (TensionTest.H:102-197): all traction, then u_x fixed
    on x-lo, u_x (disp) or t_x (trac) loaded on x-hi, u_y fixed on y-lo and
    u_z fixed on z-lo."""
    kw = {mode: 0.3}
    bt, bv = B.TensionTest("uniaxial_stress", **kw).tables()
    xload = B.DISPLACEMENT if mode == "disp" else B.TRACTION
    assert _regions(bt, 0, B.DISPLACEMENT) == (XLO | XHI if xload == B.DISPLACEMENT else XLO)
    assert _regions(bt, 1, B.DISPLACEMENT) == YLO
    assert _regions(bt, 2, B.DISPLACEMENT) == ZLO
    assert {B.FACES[f] for f in range(26) if bv[f, 0] != 0} == XHI
    assert np.all(bv[[B.FACE[f] for f in XHI], 0] == 0.3)


def test_tension_uniaxial_strain():
    """uniaxial_strain (TensionTest.H:198-298): u_x fixed / pulled on the x
    ends, u_y on both y sides, u_z on both z sides, traction elsewhere."""
    bt, bv = B.TensionTest("uniaxial_strain", disp=0.1).tables()
    assert _regions(bt, 0, B.DISPLACEMENT) == XLO | XHI
    assert _regions(bt, 1, B.DISPLACEMENT) == YLO | YHI
    assert _regions(bt, 2, B.DISPLACEMENT) == ZLO | ZHI
    assert {B.FACES[f] for f in range(26) if bv[f, 0] != 0} == XHI


def test_tension_argument_errors():
    with pytest.raises(ValueError):
        B.TensionTest("uniaxial_stress", disp=0.1, trac=0.1)
    with pytest.raises(ValueError):
        B.TensionTest("uniaxial_stress")
    with pytest.raises(ValueError):
        B.TensionTest("biaxial", disp=0.1)

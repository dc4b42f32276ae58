"""Boundary-condition tables for the nodal elastic operator.

Host-side mirror of ``BC::Operator::Elastic::Constant`` and
``BC::Operator::Elastic::TensionTest`` of the reference
(src/BC/Operator/Elastic/Constant.H, src/BC/Operator/Elastic/TensionTest.H).
A boundary condition is a table of 26 regions (6 faces, 12 edges, 8 corners)
by 3 displacement components; each entry has a type (displacement, traction,
neumann, periodic, none) and a constant value.  The region order is the
reference's ``Face`` enum (src/BC/Operator/Elastic/Elastic.H:35-43); the C ABI
(include/agb.h) takes the two tables as ``int[26][3]`` and ``double[26][3]``.
"""
import numpy as np

DISPLACEMENT, TRACTION, PERIODIC, NEUMANN, NONE = 0, 1, 2, 3, 4

FACES = [
    "xlo", "ylo", "zlo", "xhi", "yhi", "zhi",
    "ylozlo", "ylozhi", "yhizlo", "yhizhi",
    "zloxlo", "zloxhi", "zhixlo", "zhixhi",
    "xloylo", "xloyhi", "xhiylo", "xhiyhi",
    "xloylozlo", "xloylozhi", "xloyhizlo", "xloyhizhi",
    "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi",
]
FACE = {name: i for i, name in enumerate(FACES)}

# type names accepted by Constant::Parse (Constant.H:441-447)
TYPE_NAMES = {
    "displacement": DISPLACEMENT, "disp": DISPLACEMENT,
    "neumann": NEUMANN,
    "traction": TRACTION, "trac": TRACTION,
    "periodic": PERIODIC,
}


class Constant:
    """26x3 type/value table; default is zero displacement everywhere
    (Constant.H:36-45)."""

    def __init__(self, types=None, values=None):
        self.type = np.full((26, 3), DISPLACEMENT, dtype=np.int32)
        self.val = np.zeros((26, 3), dtype=np.float64)
        for face, t in (types or {}).items():
            self.set_type(face, t)
        for face, v in (values or {}).items():
            self.set_val(face, v)

    def set_type(self, face, types):
        f = FACE[face] if isinstance(face, str) else int(face)
        if isinstance(types, str):
            types = types.split()
        for d in range(3):
            t = types[d]
            self.type[f, d] = TYPE_NAMES[t] if isinstance(t, str) else int(t)

    def set_val(self, face, vals):
        f = FACE[face] if isinstance(face, str) else int(face)
        if isinstance(vals, str):
            vals = [float(v) for v in vals.split()]
        self.val[f, :] = np.asarray(vals, dtype=np.float64)

    def set(self, face, direction, bctype, value):
        """``Constant::Set(face, direction, type, value)`` (Constant.H:53-61)."""
        f = FACE[face] if isinstance(face, str) else int(face)
        self.type[f, direction] = TYPE_NAMES[bctype] if isinstance(bctype, str) else int(bctype)
        self.val[f, direction] = float(value)

    @classmethod
    def parse(cls, kv):
        """Build from ``type.<face>`` / ``val.<face>`` keys as Constant::Parse
        reads them (Constant.H:439-648)."""
        bc = cls()
        for k, v in kv.items():
            kind, face = k.split(".", 1)
            if kind == "type":
                bc.set_type(face, v)
            elif kind == "val":
                bc.set_val(face, v)
            else:
                raise KeyError(k)
        return bc

    def tables(self):
        return np.ascontiguousarray(self.type), np.ascontiguousarray(self.val)


class TensionTest(Constant):
    """``BC::Operator::Elastic::TensionTest`` (TensionTest.H:48-306) for the
    three 3D modes; loading is either ``disp`` or ``trac``."""

    def __init__(self, type="uniaxial_stress_clamp", disp=None, trac=None):
        super().__init__()
        if disp is not None and trac is not None:
            raise ValueError("Cannot specify both trac and disp")
        if disp is None and trac is None:
            raise ValueError("You must specify either trac or disp")
        mode_disp = disp is not None
        disp = 0.0 if disp is None else float(disp)
        trac = 0.0 if trac is None else float(trac)
        T, V = self.type, self.val
        F = FACE
        if type == "uniaxial_stress_clamp":
            for f in ["xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo",
                      "xhiyhizhi"]:
                V[F[f], 0] = disp
            for f in ["ylo", "yhi", "zlo", "zhi", "ylozlo", "yhizlo", "ylozhi", "yhizhi"]:
                T[F[f], :] = TRACTION
        elif type == "uniaxial_kolsky":
            for f in ["xlo", "xloylo", "xloyhi"]:
                V[F[f], 0] = disp
            for f in ["ylo", "yhi"]:
                T[F[f], :] = TRACTION
        elif type in ("uniaxial_stress", "uniaxial_strain"):
            T[:, :] = TRACTION
            for f in ["xlo", "xloylo", "xloyhi", "zloxlo", "zhixlo", "xloylozlo", "xloylozhi", "xloyhizlo",
                      "xloyhizhi"]:
                T[F[f], 0] = DISPLACEMENT
            xhi = ["xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo", "xhiyhizhi"]
            if type == "uniaxial_strain" or mode_disp:
                for f in xhi:
                    T[F[f], 0] = DISPLACEMENT
                    V[F[f], 0] = disp
            else:
                for f in xhi:
                    T[F[f], 0] = TRACTION
                    V[F[f], 0] = trac
            ylo = ["ylo", "xloylo", "xhiylo", "ylozlo", "ylozhi", "xloylozlo", "xloylozhi", "xhiylozlo", "xhiylozhi"]
            for f in ylo:
                T[F[f], 1] = DISPLACEMENT
            zlo = ["zlo", "ylozlo", "yhizlo", "zloxlo", "zloxhi", "xloylozlo", "xloyhizlo", "xhiylozlo", "xhiyhizlo"]
            for f in zlo:
                T[F[f], 2] = DISPLACEMENT
            if type == "uniaxial_strain":
                for f in ["yhi", "xloyhi", "xhiyhi", "yhizlo", "yhizhi", "xloyhizlo", "xloyhizhi", "xhiyhizlo",
                          "xhiyhizhi"]:
                    T[F[f], 1] = DISPLACEMENT
                for f in ["zhi", "ylozhi", "yhizhi", "zhixlo", "zhixhi", "xloylozhi", "xloyhizhi", "xhiylozhi",
                          "xhiyhizhi"]:
                    T[F[f], 2] = DISPLACEMENT
        else:
            raise ValueError("Unknown BC type " + str(type))

"""Boundary-condition tables for the nodal elastic operator.

Host-side mirror of ``BC::Operator::Elastic::Constant`` and
``BC::Operator::Elastic::TensionTest`` of the reference
(src/BC/Operator/Elastic/Constant.H, src/BC/Operator/Elastic/TensionTest.H).
A boundary condition is a table of 26 regions (6 faces, 12 edges, 8 corners)
by 3 displacement components; each entry has a type (displacement, traction,
neumann, periodic, none) and a constant value.  The region order is the
reference's ``Face`` enum (src/BC/Operator/Elastic/Elastic.H:35-43); the C ABI
(include/agb.h) takes the two tables as ``int[26][3]`` and ``double[26][3]``.

Values may depend on time, as the reference's values are
``Numeric::Interpolator::Linear`` objects evaluated at the BC's time
(``SetTime``, src/BC/Operator/Elastic/Elastic.H:49; Constant.H:189): a value
is a number or an interpolator string ``(t1,t2,...:v1,v2,...)``, and
``tables(time)`` returns the values at that time.
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


class Linear:
    """``Numeric::Interpolator::Linear<Set::Scalar>``
    (src/Numeric/Interpolator/Linear.H:56-157): piecewise-linear in time.

    Built from a number (constant) or from a string ``(t1,...,tn:v1,...,vn)``
    (Linear.H:73-111; unitless values only).  A string with any of ``( , : )``
    must have both parentheses and the colon, equally many times and values,
    and non-decreasing times, else ``ValueError`` (the reference aborts).
    Evaluation follows Linear.H:121-157 exactly, including its search start
    for uniformly spaced times: below the first time the first value, in an
    interval the linear interpolant, and otherwise (past the last time, or an
    interval the uniform-spacing guess skipped when the spacing is not
    uniform) the last value."""

    def __init__(self, spec=0.0):
        if isinstance(spec, Linear):
            self.times, self.values = list(spec.times), list(spec.values)
            return
        if not isinstance(spec, str):
            self.times, self.values = [0.0], [float(spec)]
            return
        s = spec.strip()
        if any(c in s for c in "(:),"):
            if "(" not in s or ")" not in s:
                raise ValueError("Mismatched parentheses while trying to parse " + spec)
            if ":" not in s:
                raise ValueError("Missing : in interpolator while trying to parse " + spec)
            s = s.replace("(", "").replace(")", "")
            st, sv = s.split(":")[:2]
            ts, vs = st.split(","), sv.split(",")
            if len(ts) != len(vs):
                raise ValueError("Mismatched number of time values vs array values while trying to parse " + spec)
            self.times, self.values = [], []
            for i, (t, v) in enumerate(zip(ts, vs)):
                self.times.append(float(t))
                if i > 0 and self.times[i] < self.times[i - 1]:
                    raise ValueError("Time series must monotonically increase - error while trying to parse " + spec)
                self.values.append(float(v))
        else:
            self.times, self.values = [0.0], [float(s)]

    def __call__(self, t):
        tp, vp = self.times, self.values
        if len(vp) == 1:
            return vp[0]
        if t < tp[0]:
            return vp[0]
        start = int((t - tp[0]) / (tp[1] - tp[0])) - 1
        start = min(max(start, 0), len(tp) - 2)
        for i in range(start, len(tp) - 1):
            if tp[i] <= t <= tp[i + 1]:
                return vp[i] + (t - tp[i]) * (vp[i + 1] - vp[i]) / (tp[i + 1] - tp[i])
        return vp[-1]

    @property
    def constant(self):
        return len(self.values) == 1


class Constant:
    """26x3 type/value table; default is zero displacement everywhere
    (Constant.H:36-45).  ``val`` holds the values at the current time
    (``set_time``); entries given as interpolators are re-evaluated there."""

    def __init__(self, types=None, values=None):
        self.type = np.full((26, 3), DISPLACEMENT, dtype=np.int32)
        self.val = np.zeros((26, 3), dtype=np.float64)
        self.time = 0.0
        self._interp = {}
        for face, t in (types or {}).items():
            self.set_type(face, t)
        for face, v in (values or {}).items():
            self.set_val(face, v)

    def _put(self, f, d, value):
        lin = Linear(value)
        if lin.constant:
            self._interp.pop((f, d), None)
        else:
            self._interp[(f, d)] = lin
        self.val[f, d] = lin(self.time)

    def set_time(self, time):
        """``SetTime`` (src/BC/Operator/Elastic/Elastic.H:49): the time at
        which interpolated values are evaluated."""
        self.time = float(time)
        for (f, d), lin in self._interp.items():
            self.val[f, d] = lin(self.time)

    def set_type(self, face, types):
        f = FACE[face] if isinstance(face, str) else int(face)
        if isinstance(types, str):
            types = types.split()
        for d in range(3):
            t = types[d]
            self.type[f, d] = TYPE_NAMES[t] if isinstance(t, str) else int(t)

    def set_val(self, face, vals):
        """Values of one region, as numbers or interpolator strings; a string
        holds the three whitespace-separated entries (Constant.H:563-648)."""
        f = FACE[face] if isinstance(face, str) else int(face)
        if isinstance(vals, str):
            vals = vals.split()
        for d in range(3):
            self._put(f, d, vals[d])

    def set(self, face, direction, bctype, value):
        """``Constant::Set(face, direction, type, value)`` (Constant.H:53-61)."""
        f = FACE[face] if isinstance(face, str) else int(face)
        self.type[f, direction] = TYPE_NAMES[bctype] if isinstance(bctype, str) else int(bctype)
        self._put(f, direction, value)

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

    def tables(self, time=None):
        """(type int32[26][3], value float64[26][3]) for the C ABI, the values
        at ``time`` (set with ``set_time``) when it is given."""
        if time is not None:
            self.set_time(time)
        return np.ascontiguousarray(self.type), np.ascontiguousarray(self.val)


class TensionTest(Constant):
    """``BC::Operator::Elastic::TensionTest`` (TensionTest.H:48-306): the
    modes uniaxial_stress_clamp, uniaxial_kolsky, uniaxial_stress and
    uniaxial_strain; loading is either ``disp`` or ``trac``, each a number or
    an interpolator string in time (TensionTest.H:56-68)."""

    def __init__(self, type="uniaxial_stress_clamp", disp=None, trac=None):
        super().__init__()
        if disp is not None and trac is not None:
            raise ValueError("Cannot specify both trac and disp")
        if disp is None and trac is None:
            raise ValueError("You must specify either trac or disp")
        mode_disp = disp is not None
        disp = Linear(0.0 if disp is None else disp)
        trac = Linear(0.0 if trac is None else trac)
        T = self.type
        F = FACE
        if type == "uniaxial_stress_clamp":
            for f in ["xhi", "xhiylo", "xhiyhi", "zloxhi", "zhixhi", "xhiylozlo", "xhiylozhi", "xhiyhizlo",
                      "xhiyhizhi"]:
                self._put(F[f], 0, disp)
            for f in ["ylo", "yhi", "zlo", "zhi", "ylozlo", "yhizlo", "ylozhi", "yhizhi"]:
                T[F[f], :] = TRACTION
        elif type == "uniaxial_kolsky":
            for f in ["xlo", "xloylo", "xloyhi"]:
                self._put(F[f], 0, disp)
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
                    self._put(F[f], 0, disp)
            else:
                for f in xhi:
                    T[F[f], 0] = TRACTION
                    self._put(F[f], 0, trac)
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

"""Problem set-ups shared by the parity tests (inputs only, no solver)."""
import numpy as np

from alamo_gb300 import bc as B
from alamo_gb300 import synth

SEED = 20261203


def c1(n=33):
    """Config 1: isotropic matrix lambda=mu=1, centred inclusion r=0.25 with
    lambda=mu=10 and eigenstrain 0.01 I, zero displacement on all faces."""
    C, F0, dx = synth.inclusion_iso(n)
    return C, F0, B.Constant(), dx


def voronoi_clamp(n=33, nseeds=64, seed=7, disp=0.01):
    """Config 2 shape: cubic Voronoi polycrystal, uniaxial_stress_clamp."""
    C, dx = synth.voronoi_cubic(n, nseeds, seed=seed)
    return C, None, B.TensionTest("uniaxial_stress_clamp", disp=disp), dx


def random_bc(seed):
    """Every region gets a random type among displacement / traction /
    neumann and a random value: exercises all 26 x 3 boundary rows."""
    rng = np.random.default_rng(seed)
    bc = B.Constant()
    bc.type[:, :] = rng.choice([B.DISPLACEMENT, B.TRACTION, B.NEUMANN], size=(26, 3))
    bc.val[:, :] = rng.uniform(-1, 1, size=(26, 3))
    return bc


def random_field(shape, seed=SEED):
    return synth.uniform(seed, shape)


def iso_as_mm(C):
    """The isotropic tensor written as 21 major-minor entries."""
    lam, mu = C[..., 0], C[..., 1]
    out = np.zeros(C.shape[:-1] + (21,))
    # pair order (00,01,02,11,12,22); C_iijj = lam, C_iiii = lam + 2 mu, C_ijij = mu
    ut = {}
    c = 0
    for a in range(6):
        for b in range(a, 6):
            ut[(a, b)] = c
            c += 1
    diag_pairs = [0, 3, 5]
    shear_pairs = [1, 2, 4]
    for a in diag_pairs:
        for b in diag_pairs:
            if a <= b:
                out[..., ut[(a, b)]] = lam + (2 * mu if a == b else 0)
    for a in shear_pairs:
        out[..., ut[(a, a)]] = mu
    return out

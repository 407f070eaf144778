"""Problems shared by the refshim tests and the reference golden fixtures."""
import numpy as np

from nlmech_gb300 import abi, configs
from nlmech_gb300.decks import BC, Crack


def fracture_plate():
    """48 x 48 plate, horizon 3h, 12 mm pre-crack, +-0.5 m/s: the crack grows
    within 300 steps."""
    return configs.rnp_plate(48, 1e-3, 3, 0.012, 0.5, 2e-8, 300, seed=7)


def loads_nofail_plate():
    """Force BCs (linear and sin in time, constant and linear_y in space), a
    sin-in-time displacement BC, a computed no-fail layer and the linear
    influence function."""
    p = configs.rnp_plate(40, 1e-3, 3, 0.01, 0.3, 2e-8, 200, seed=11)
    p.material.influence_type = 1
    p.material.influence_params = []
    p.fbc = [BC(region="rectangle", x1=0.0, x2=0.004, y1=0.0, y2=0.04, direction=[1],
                time_fn="linear", time_params=[1.0], spatial_fn="constant",
                spatial_params=[-2e12]),
             BC(region="rectangle", x1=0.0, x2=0.002, y1=0.0, y2=0.04, direction=[1, 2],
                time_fn="sin", time_params=[1.0, 2e4], spatial_fn="linear_y",
                spatial_params=[1e14])]
    p.ubc.append(BC(region="rectangle", x1=0.036, x2=0.041, y1=0.01, y2=0.03, direction=[1],
                    time_fn="sin", time_params=[1e-7, 5e4], spatial_fn="constant",
                    spatial_params=[1.0]))
    p.no_fail = abi.NOFAIL_COMPUTE
    p.no_fail_tol = 2e-3
    return p


def cube3d(n=12, seed=5):
    """3-D RNPBond cube n^3 (h = 1 mm, horizon 3h), no displacement BC,
    seeded random initial velocities of +-0.5 m/s in every direction."""
    x, vol = configs.grid3d(n, n, n, 1e-3, seed=seed)
    p = configs.rnp_plate(8, 1e-3, 3, 0.0, 0.1, 2e-8, 100)
    p.dim = 3
    p.x, p.volume = x, vol
    p.horizon = 3e-3
    p.cracks = []
    p.ubc = []
    rng = np.random.default_rng(seed)
    p.v0 = rng.uniform(-0.5, 0.5, size=(x.shape[0], 3))
    return p


def contact_plate():
    """32 x 32 plate with a pre-crack, no boundary loads, seeded random
    initial velocities of +-2 m/s: bonds break and broken-bond nodes come
    within the contact radius, so the No_Penetration contact force acts."""
    p = configs.rnp_plate(32, 1e-3, 3, 0.008, 0.0, 2e-8, 300, seed=3)
    p.ubc = []
    rng = np.random.default_rng(4)
    p.v0 = np.zeros((p.n, 3))
    p.v0[:, :2] = rng.uniform(-2.0, 2.0, size=(p.n, 2))
    p.material.apply_contact = True
    return p


def timed_crack_plate():
    """40 x 40 plate with a pre-crack and three timed cracks (Activation_Time):
    one at t = 0 (cut after the first step), two at 3e-7 s (the first cut
    after step 16, the second one step later: one crack per step)."""
    p = configs.rnp_plate(40, 1e-3, 3, 0.008, 0.3, 2e-8, 200, seed=5)
    W = 0.04
    p.cracks += [
        Crack(kind="edge", orientation=1, pb=(0.004, 0.3 * W), pt=(0.016, 0.3 * W),
              activation_time=3e-7),
        Crack(kind="edge", orientation=-1, pb=(0.7 * W, 0.006), pt=(0.7 * W, 0.018),
              activation_time=3e-7),
        Crack(kind="edge", orientation=1, pb=(0.022, 0.75 * W), pt=(0.034, 0.75 * W),
              activation_time=0.0),
    ]
    return p


def reaction_plate():
    """40 x 40 plate at h = 1 m (horizon 3 m), pulled at 1e-4 m/s: the
    reaction-force layer below the top boundary carries bond forces, and at
    this scale the orientation test of the reference's doLinesIntersect
    (an int-truncated cross product) separates the two sides of the line."""
    return configs.rnp_plate(40, 1.0, 3, 8.0, 1e-4, 2e-5, 200, seed=2)


def nofail_regions_plate():
    """The growing-crack plate with a stored no-fail layer and the
    No_Fail_Region list: a circle around the right crack tip and a rectangle
    across the left one, whose bonds never break."""
    p = fracture_plate()
    p.no_fail = abi.NOFAIL_DATA
    p.no_fail_tol = 1.5e-3
    p.nofail_regions = [("Circle", [0.03, 0.024, 0.0, 4e-3]),
                        ("Rectangle", [0.006, 0.02, 0.014, 0.028])]
    return p


def force_functions_plate():
    """Force_BC spatial functions hat_x, hat_y and line_load (from either
    end) on a 40 x 40 plate."""
    p = configs.rnp_plate(40, 1e-3, 3, 0.01, 0.2, 2e-8, 200, seed=13)
    lin = dict(time_fn="linear", time_params=[1.0])
    p.fbc = [BC(region="rectangle", x1=0.005, x2=0.035, y1=0.030, y2=0.036, direction=[2],
                spatial_fn="hat_x", spatial_params=[4e13], **lin),
             BC(region="rectangle", x1=0.0, x2=0.004, y1=0.004, y2=0.036, direction=[1],
                spatial_fn="hat_y", spatial_params=[-3e13], **lin),
             BC(region="rectangle", x1=0.036, x2=0.04, y1=0.004, y2=0.036, direction=[1],
                spatial_fn="line_load", spatial_params=[1.0], time_fn="linear",
                time_params=[2e13]),
             BC(region="rectangle", x1=0.005, x2=0.035, y1=0.004, y2=0.01, direction=[2],
                spatial_fn="line_load", spatial_params=[-1.0], time_fn="linear",
                time_params=[-2e13])]
    return p


def angled_regions_plate():
    """Angled_Rectangle regions: a Displacement_BC strip turned by 0.3 rad
    and a Force_BC patch turned by -0.2 rad, plus a Force_BC cuboid (a 3-D
    box test on a 2-D mesh, z = 0 inside)."""
    p = configs.rnp_plate(40, 1e-3, 3, 0.01, 0.2, 2e-8, 200, seed=17)
    p.ubc.append(BC(region="angled_rectangle", x1=0.002, y1=0.012, x2=0.012, y2=0.020,
                    theta=0.3, direction=[1], time_fn="linear", time_params=[-0.05]))
    p.fbc = [BC(region="angled_rectangle", x1=0.025, y1=0.012, x2=0.036, y2=0.016, theta=-0.2,
                direction=[1, 2], time_fn="linear", time_params=[1.0],
                spatial_params=[3e13]),
             BC(region="cuboid", x1=0.015, y1=0.004, z1=-1.0, x2=0.025, y2=0.008, z2=1.0,
                direction=[2], time_fn="sin", time_params=[2e13, 3e4])]
    return p


def gaussian_plate():
    """The growing-crack plate with the Gaussian influence function
    J(r) = alpha exp(-r^2 / beta) at its default parameters (beta = 0.2,
    alpha making the d-th moment one; influenceFn.h:278-307)."""
    p = fracture_plate()
    p.material.influence_type = 2
    p.material.influence_params = []
    return p


def gaussian_params_plate():
    """The Gaussian influence function with parameters from the deck
    (alpha = 1.5, beta = 0.35; influenceFn.h:302-305), on the plate with
    force BCs and a computed no-fail layer."""
    p = loads_nofail_plate()
    p.material.influence_type = 2
    p.material.influence_params = [1.5, 0.35]
    return p


# name -> (problem, Verlet steps) of the committed reference outputs
# (tests/golden/rnp_ref_<name>.npz)
GOLDEN_CASES = {
    "fracture_plate": (fracture_plate, 300),
    "loads_nofail_plate": (loads_nofail_plate, 200),
    "cube3d": (cube3d, 100),
    "contact_plate": (contact_plate, 300),
    "timed_crack_plate": (timed_crack_plate, 200),
    "reaction_plate": (reaction_plate, 200),
    "nofail_regions_plate": (nofail_regions_plate, 300),
    "force_functions_plate": (force_functions_plate, 200),
    "angled_regions_plate": (angled_regions_plate, 200),
    "gaussian_plate": (gaussian_plate, 300),
    "gaussian_params_plate": (gaussian_params_plate, 200),
}

"""Host-side set-up of a DVM run: velocity grids, molecule constants, cross-section,
initial distributions and normal-shock end states.

This is init-time host logic (the reference does it once in initialize_solver,
solver/dvm_solver.f90:92-229); the GPU kernels consume its output through the C ABI.
Citations are to aarthisekaran11/2D_DVM_microflows, software/trunk/src.
"""
import math

import numpy as np

PI_REFERENCE = 3.1459265358979323  # utils/constants.f90:30 (sic)
PI_EXACT = math.pi
KB_REFERENCE = 1.3805e-23           # utils/constants.f90:31, Boltzmann's constant [J/K]


def pi_value(pi_mode):
    return PI_EXACT if pi_mode == 1 else PI_REFERENCE


# --------------------------------------------------------------------------------------
def uniform_axis(n, vmin, vmax):
    """generate_uniform_grid (grid/velocity_grid.f90:631-651): v_min + i*(v_max-v_min)/(n-1),
    evaluated in the same order."""
    i = np.arange(n, dtype=np.float64)
    return vmin + i * (vmax - vmin) / float(n - 1)


def node_volumes(a):
    """compute_beta (grid/velocity_grid.f90:486-540): half-distances to the neighbours,
    full spacing at the two ends."""
    b = np.empty_like(a)
    b[0] = a[1] - a[0]
    b[-1] = a[-1] - a[-2]
    b[1:-1] = (a[2:] - a[1:-1]) / 2.0 + (a[1:-1] - a[:-2]) / 2.0
    return b


class VelocityGrid:
    """Node coordinates per axis; v = i + nx*(j + ny*k)."""

    def __init__(self, x, y=None, z=None):
        self.x = np.ascontiguousarray(x, dtype=np.float64)
        self.y = np.ascontiguousarray(self.x if y is None else y, dtype=np.float64)
        self.z = np.ascontiguousarray(self.x if z is None else z, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.x), len(self.y), len(self.z)
        self.nv = self.nx * self.ny * self.nz
        self.bx, self.by, self.bz = (node_volumes(self.x), node_volumes(self.y),
                                     node_volumes(self.z))

    @classmethod
    def uniform(cls, n, vmin, vmax):
        ax = uniform_axis(n, vmin, vmax)
        return cls(ax, ax.copy(), ax.copy())

    def mesh(self):
        """(X, Y, Z, beta3) flattened in the f[v] order, beta3 = bx*by*bz."""
        Z, Y, X = np.meshgrid(self.z, self.y, self.x, indexing="ij")
        BZ, BY, BX = np.meshgrid(self.bz, self.by, self.bx, indexing="ij")
        return (X.ravel(), Y.ravel(), Z.ravel(), (BX * BY * BZ).ravel())

    def beta3_min(self):
        return float((self.bx[:, None, None] * self.by[None, :, None] *
                      self.bz[None, None, :]).min())


# --------------------------------------------------------------------------------------
def gamma_reference(x, pi_mode=0):
    """gamma_calculator (utils/math_utils.f90:79-135): Lanczos approximation (g = 7, nine
    coefficients, as published with the GNU Scientific Library), with the reference pi."""
    pi = pi_value(pi_mode)
    coef = [0.99999999999980993, 676.5203681218851, -1259.1392167224028,
            771.32342877765313, -176.61502916214059, 12.507343278686905,
            -0.13857109526572012, 9.9843695780195716e-6, 1.5056327351493116e-7]
    if x < 0.5:
        return pi / (math.sin(pi * x) * gamma_reference(1.0 - x, pi_mode))
    x = x - 1.0
    y = coef[0]
    for i in range(1, 9):
        y = y + coef[i] / (x + float(i))
    z = x + 7.0 + 0.5
    return math.sqrt(2.0 * pi) * z ** (x + 0.5) * math.exp(-z) * y


CSECTION_CLARKE, CSECTION_BIRD, CSECTION_VKI = 1, 2, 3
CSECTION_HS, CSECTION_PM, CSECTION_VHS, CSECTION_VSS = 1, 2, 3, 4

def _real4(x):
    """The table's diameters and masses are default-real (single precision) literals in the
    reference; keep their float32 rounding."""
    return float(np.float32(x))


# Monatomic molecule table (input_output/species_data.f90:255-304), SI units.
SPECIES = {
    "He": dict(diam=_real4(2.33e-10), mass=_real4(6.65e-27), omega=0.66, alpha=1.31),
    "Ne": dict(diam=_real4(2.77e-10), mass=_real4(33.5e-27), omega=0.66, alpha=1.31),
    "Ar": dict(diam=_real4(4.17e-10), mass=_real4(66.3e-27), omega=0.81, alpha=1.40,
               viscosity=_real4(2.75e-5), T_viscosity=380.0),
    "Xe": dict(diam=_real4(5.74e-10), mass=_real4(218.e-27), omega=0.85, alpha=1.44),
}


def molecule(species="Ar", csection_method=CSECTION_HS, ref_species=None):
    """Scaled molecule constants (set_molecule_constants, species_data.f90:155-229) with the
    cross-section model override (get_molecule_info :503-521). Single species: it is its own
    reference, so mass = diam = 1."""
    s = SPECIES[species]
    ref = SPECIES[ref_species or species]
    omega, alpha = s["omega"], s["alpha"]
    if csection_method == CSECTION_HS:
        omega, alpha = 0.5, 1.0
    elif csection_method == CSECTION_PM:
        omega, alpha = 1.0, 1.0
    elif csection_method == CSECTION_VHS:
        alpha = 1.0
    return dict(mass=s["mass"] / ref["mass"], diam=s["diam"] / ref["diam"],
                omega=omega, alpha=alpha)


def reference_values(dens, temp, species="Ar", Kn=1.0, pi_mode=0):
    """The dimensional reference values of a run (set_scaling_parameters,
    solver/scaling.f90:118-148, and the derived ones of write_reference_values_to_file
    :203-237): reference speed sqrt(2 kb T/m), cross-section pi d^2, length 1/(Kn n sigma),
    time L/c, pressure 2 kb n T, heat flux m c^3, energy m c^2 (SI units), for the reference
    species' single-precision mass and diameter."""
    s = SPECIES[species]
    m, d = s["mass"], s["diam"]
    c = math.sqrt(2.0 * KB_REFERENCE * temp / m)
    sigma = pi_value(pi_mode) * d * d
    L = 1.0 / (Kn * dens * sigma)
    return {"Mass": m, "Diameter": d, "Cross-section": sigma, "Density": dens,
            "Temperature": temp, "Speed": c, "Pressure": 2.0 * KB_REFERENCE * dens * temp,
            "Heat Flux": m * c * c * c, "Energy": m * c * c, "Flow Knudsen number": Kn,
            "Characteristic length scale": L, "Time scale": L / c}


def cross_section(mol, csection_coeff=CSECTION_BIRD, pi_mode=0, viscosity=None,
                  temp_visc=None):
    """calculate_cross_section (solver/scaling.f90:163-201) for a like-species pair."""
    m = mol["mass"]
    m_red = m * m / (m + m)
    d = mol["diam"]
    omega = 0.5 * (mol["omega"] + mol["omega"])
    sigma_vhs = 0.25 * (d + d) * (d + d)
    if csection_coeff == CSECTION_CLARKE:
        return sigma_vhs
    if csection_coeff == CSECTION_BIRD:
        return sigma_vhs * m_red ** (0.5 - omega) / gamma_reference(2.5 - omega, pi_mode)
    if csection_coeff == CSECTION_VKI:
        g = gamma_reference(4.5 - omega, pi_mode)
        return (3.32335097045 * m_red ** (1.0 - omega) * temp_visc ** omega) / (g * viscosity)
    raise ValueError("invalid csection_coeff %r" % (csection_coeff,))


# --------------------------------------------------------------------------------------
def maxwellian(grid, dens, u, v, w, temp, mass=1.0, pi_mode=0, renormalise=True):
    """Discrete Maxwellian times the node volume, as initialize_dist_func builds it
    (conditions/initial_conditions.f90:480-617): n (m/(pi T))^{3/2} exp(-m|c-u|^2/T) beta3,
    then scaled so that sum(f) = n."""
    pi = pi_value(pi_mode)
    X, Y, Z, B3 = grid.mesh()
    opt = mass / (pi * temp)
    coeff = dens * math.sqrt(opt * opt * opt)
    csq = (X - u) ** 2 + (Y - v) ** 2 + (Z - w) ** 2
    f = coeff * np.exp(-csq * mass / temp) * B3
    if renormalise:
        s = f.sum()
        if s > 0:
            f = (dens / s) * f
    return f


def bkw_xk(time):
    """The BKW shape parameter K at time t (collision times of a Maxwell gas), from 3/5 at
    t = 0 to 1: generate_bkw (conditions/initial_conditions.f90:693-695)."""
    return 1.0 - 0.4 * math.exp(-time / 6.0)


def bkw(grid, dens, temp, time=0.0, mass=1.0, u=0.0, v=0.0, w=0.0, pi_mode=0,
        renormalise=True):
    """Discrete Bobylev-Krook-Wu distribution times the node volume (compute_bkw,
    dist_funcs/dist_func.f90:374-401, as generate_bkw uses it): with K = bkw_xk(time),
    n/2 (m/(pi T))^{3/2} K^{-5/2} (5K - 3 + 2(1-K) m|c-u|^2/(K T)) exp(-m|c-u|^2/(K T)),
    scaled so that sum(f) = n. The exact solution of the isotropic Maxwell-molecule
    Boltzmann equation with time in units of the inverse collision frequency."""
    pi = pi_value(pi_mode)
    X, Y, Z, B3 = grid.mesh()
    xk = bkw_xk(time)
    opt = mass / (pi * temp)
    norm = 0.5 * dens * math.sqrt(opt * opt * opt) * xk ** (-2.5)
    csq = (X - u) ** 2 + (Y - v) ** 2 + (Z - w) ** 2
    f = norm * (5.0 * xk - 3.0 + 2.0 * (1.0 - xk) * csq * mass / (xk * temp)) * \
        np.exp(-csq * mass / (xk * temp)) * B3
    if renormalise:
        s = f.sum()
        if s != 0:
            f = (dens / s) * f
    return f


def bimodal(grid, w1=0.5, T1=1.0, u1=1.0, w2=0.5, T2=3.0, u2=-1.0, mass=1.0, pi_mode=0):
    """Sum of two renormalised Maxwellians with x-drifts (the 0-D relaxation state)."""
    return (w1 * maxwellian(grid, 1.0, u1, 0.0, 0.0, T1, mass, pi_mode) +
            w2 * maxwellian(grid, 1.0, u2, 0.0, 0.0, T2, mass, pi_mode))


def normal_shock(mach, gamma=5.0 / 3.0, T_up=1.0, n_up=1.0, mass=1.0):
    """Stationary normal shock (conditions/shock_conditions.f90:54-171). The flow runs in -x:
    upstream at the right end, u_up < 0. Returns (upstream, downstream) dicts of n, u, T."""
    a_up = math.sqrt(gamma * T_up / (2.0 * mass))
    u_up = -mach * a_up
    M = mach
    T_ratio = ((1.0 + 2.0 * gamma * (M * M - 1.0) / (gamma + 1.0)) *
               (2.0 + (gamma - 1.0) * M * M) / ((gamma + 1.0) * M * M))
    dens_ratio = (gamma + 1.0) * M * M / (2.0 + (gamma - 1.0) * M * M)
    M_down = math.sqrt((1.0 + 0.5 * (gamma - 1.0) * M * M) /
                       (gamma * M * M - 0.5 * (gamma - 1.0)))
    T_down = T_ratio * T_up
    a_down = math.sqrt(gamma * T_down / (2.0 * mass))
    u_down = -a_down * M_down
    return (dict(n=n_up, u=u_up, T=T_up),
            dict(n=n_up * dens_ratio, u=u_down, T=T_down))


def shock_profile(grid, nx_space, dx, mach, width, mass=1.0, pi_mode=0):
    """1-D shock initial state: downstream Maxwellian on the left, upstream on the right,
    joined by tanh profiles of n, u and T (width in upstream mean free paths, the cell
    size dx in the same units). Returns (f[nx_space, nv], upstream, downstream)."""
    up, dn = normal_shock(mach, mass=mass)
    xc = (np.arange(nx_space) + 0.5) * dx
    x0 = 0.5 * nx_space * dx
    s = 0.5 * (1.0 + np.tanh((xc - x0) / width))  # 0 on the left, 1 on the right
    f = np.empty((nx_space, grid.nv))
    for c in range(nx_space):
        n = dn["n"] + (up["n"] - dn["n"]) * s[c]
        u = dn["u"] + (up["u"] - dn["u"]) * s[c]
        T = dn["T"] + (up["T"] - dn["T"]) * s[c]
        f[c] = maxwellian(grid, n, u, 0.0, 0.0, T, mass, pi_mode)
    return f, up, dn

"""The oracle's sea-level equation: a numpy restatement of GRDSolver::
SolveGeneralised (src/SeaLevel.cpp:397-736) with its forcing channels and
rotational feedback, and of the plain Anderson mixer it runs
(include/sl3dpp/detail/AndersonMixer.hpp:65-219); the nonlinear solve with
migrating shorelines, GRDSolver::SolveNonlinear (src/SeaLevel.cpp:970-1289),
and the flotation of MakeState (:279-300). Test infrastructure: the
checker the GPU solver (sl3dgpu_sle_solve) is compared with; it takes the
grid's transforms and quadrature as arguments.

Pinned to the reference's own gate (tests/TestFixtures.cpp:130-205): pyslfp's
generalised solve at lmax 32 with full rotational feedback and every load
channel, matched to 1.9e-9 on the lmax grid (the reference's bar 5e-9) and
3.7e-11 on a grid of twice the bandwidth (tests/test_sle_fixture.py). The
structural identities of tests/TestSeaLevel.cpp:135-206 (the rigid-earth
eustatic limit, the ocean gaining the mass the load lost) are checked too.
"""

from __future__ import annotations

import numpy as np


class AndersonMixer:
    """AndersonMixer::Update (AndersonMixer.hpp:65-219): the first call takes
    the image, later ones the least-squares mix of `memory` difference columns
    (Gram matrix by columns, minimum-norm solve with the machine-precision cut
    of dgelss's rcond < 0)."""

    def __init__(self, memory: int):
        self.memory = memory
        self.count = 0
        self.slot = 0
        self.x_prev = None

    def update(self, x: np.ndarray, gx: np.ndarray) -> np.ndarray:
        if self.memory <= 0:
            return gx.copy()
        if self.x_prev is None:
            n = x.size
            self.dG = np.zeros((self.memory, n))
            self.dF = np.zeros((self.memory, n))
            self.gram = np.zeros((self.memory, self.memory))
            self.x_prev = x.copy()
            self.f_prev = gx - x
            return gx.copy()
        slot = self.slot
        m = min(self.count + 1, self.memory)
        f = gx - x
        self.dF[slot] = f - self.f_prev
        self.dG[slot] = (x - self.x_prev) + self.dF[slot]
        self.x_prev = x.copy()
        self.f_prev = f
        column = self.dF[:m] @ self.dF[slot]
        rhs = self.dF[:m] @ f
        self.count = m
        self.slot = (slot + 1) % self.memory
        self.gram[slot, :m] = column
        self.gram[:m, slot] = column
        a = self.gram[:m, :m]
        # symmetric: singular values are the eigenvalues' magnitudes
        lam, v = np.linalg.eigh(0.5 * (a + a.T))
        cut = np.finfo(float).eps * np.max(np.abs(lam)) if lam.size else 0.0
        keep = np.abs(lam) > cut
        gamma = v[:, keep] @ ((v[:, keep].T @ rhs) / lam[keep])
        return gx - gamma @ self.dG[:m]


def _block_of(c):
    """BlockOf (src/SeaLevel.cpp:33-36): [[(2,0), cos], [0, sin]] of the (2, 1)
    real pair (ShConventions.hpp:48-54)."""
    r2 = np.sqrt(2.0)
    return np.array([[c[3].real, -r2 * c[4].real], [0.0, r2 * c[4].imag]])


def _set_block(c, b):
    """SetBlock (src/SeaLevel.cpp:38-42)."""
    r2 = np.sqrt(2.0)
    c[3] = b[0, 0]
    c[4] = complex(-b[0, 1] / r2, b[1, 1] / r2)


def _add_block(c, b):
    """AddBlock (src/SeaLevel.cpp:44-48)."""
    r2 = np.sqrt(2.0)
    c[3] += b[0, 0]
    c[4] += complex(-b[0, 1] / r2, b[1, 1] / r2)


class _RotationFactors:
    """The constructor's rotational factors (src/SeaLevel.cpp:220-247)."""

    def __init__(self, rotation, h, k, ht, kt, radius, omega, polar, equatorial, G, hc, kc, m_u, m_phi, m_c):
        pi, a, w = np.pi, radius, omega
        self.transverse = rotation == 2
        self.h2, self.k2, self.ht2, self.kt2 = h[2], k[2], ht[2], kt[2]
        self.hc, self.kc, self.mu, self.mphi, self.mc = hc, kc, m_u, m_phi, m_c
        self.rotation = np.sqrt(4.0 * pi / 15.0) * w * a * a
        self.inertia = np.sqrt(5.0 / (12.0 * pi)) * w * a ** 3 / (G * (polar - equatorial))
        self.axial_rotation = np.sqrt(16.0 * pi / 45.0) * w * a * a
        self.uniform_rotation = -np.sqrt(16.0 * pi / 9.0) * w * a * a
        self.axial_inertia = np.sqrt(5.0 / (9.0 * pi)) * w * a ** 3 / (G * polar)
        self.inverse_inertia_difference = 1.0 / (polar - equatorial)
        self.inverse_polar_inertia = 1.0 / polar
        self.trace = (4.0 / 3.0) * w / polar
        self.shell = (2.0 / 3.0) * w * a ** 4 * np.sqrt(4.0 * pi) / polar
        self.rotation_denominator = 1.0 - self.inertia * self.kt2 * self.rotation
        self.axial_rotation_denominator = (1.0 + self.axial_inertia * self.kt2 * self.axial_rotation +
                                           self.trace * self.mc * self.uniform_rotation)


def _rotation(s, load2, load0, static_disp2, static_grav2, inertia_moment, angular_momentum, displacement_load0=0.0,
              potential_load0=0.0):
    """GRDSolver::Rotation (src/SeaLevel.cpp:348-395); the load channels'
    degree-0 parts enter the axial trace and shell terms."""
    grav = s.k2 * load2 + static_grav2
    disp = s.h2 * load2 + static_disp2
    transverse = np.array([s.inertia * grav[0, 1], s.inertia * grav[1, 1]])
    axial = (-s.axial_inertia * grav[0, 0]
             - s.trace * ((s.mu + s.mphi) * load0 + s.mu * displacement_load0 + s.mphi * potential_load0
                          + inertia_moment)
             - s.shell * (load0 + potential_load0))
    transverse -= s.inverse_inertia_difference * np.asarray(angular_momentum[:2])
    axial += s.inverse_polar_inertia * angular_momentum[2]
    omega = np.zeros(3)
    if s.transverse:
        omega[:2] = transverse / s.rotation_denominator
    omega[2] = axial / s.axial_rotation_denominator
    centrifugal = np.array([[s.axial_rotation * omega[2], s.rotation * omega[0]], [0.0, s.rotation * omega[1]]])
    centrifugal0 = s.uniform_rotation * omega[2]
    return dict(omega=omega, disp2=disp + s.ht2 * centrifugal, grav2=grav + s.kt2 * centrifugal,
                centrifugal=centrifugal, centrifugal0=centrifugal0)


def solve_generalised(synthesise, expand, integrate, h, k, lt, g, water_density, radius, ocean, direct_load=None,
                      rtol=1e-9, max_iterations=1000, anderson_memory=5, direct_load_outside=None,
                      solid_surface_change=None, displacement_response=None, potential_response=None,
                      tangential_response=None, toroidal_response=None, tide=None, ht=None, kt=None, lt_tide=None,
                      rotation=0, omega=0.0, polar=0.0, equatorial=0.0, G=0.0, hc=0.0, kc=0.0, m_u=0.0, m_phi=0.0,
                      m_c=0.0, inertia_moment_change=0.0, angular_momentum_change=(0.0, 0.0, 0.0),
                      displacement_load=None, potential_load=None, tangential_traction=None, channel_numbers=None):
    """The load fixed point of the sea-level equation (SeaLevel.cpp:397-736
    with RotationalFeedback::None) for the channels the coupled Evolution3D
    closure uses, and the load channels (a displacement load, a potential
    load, a tangential traction) through their own numbers channel_numbers
    (h_u, k_u, l_u, h_phi, k_phi, l_phi, h_v, k_v, l_v; :453-502).
    synthesise(coeffs) and expand(field) are the grid's real transforms in
    the reference's (l, m >= 0) layout, integrate(field) its quadrature over
    the unit sphere."""
    h = np.asarray(h, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    lmax = h.size - 1
    degree = np.concatenate([np.full(l + 1, l) for l in range(lmax + 1)])
    ncoef = degree.size
    size = ocean.size
    out = {"uniform_shift": 0.0, "iterations": 0, "error": 0.0, "converged": True, "angular_velocity": np.zeros(3)}
    nz = lambda a: a is not None and np.max(np.abs(a)) > 0.0
    # the toroidal potential is carried, whatever else is solved (:561-563)
    toroidal = synthesise(toroidal_response) if toroidal_response is not None else np.zeros(size)
    channels = nz(displacement_load) or nz(potential_load) or nz(tangential_traction)
    any_static = (nz(displacement_response) or nz(potential_response) or nz(tide) or nz(solid_surface_change)
                  or channels)
    any_tan = nz(displacement_response) or nz(potential_response) or nz(tangential_response) or nz(tide) or channels
    if not (nz(direct_load) or nz(direct_load_outside) or any_static or any_tan):
        zeros = np.zeros(size)
        out.update(sea_level_change=zeros, displacement=zeros, potential=zeros, tangential_potential=zeros,
                   toroidal_potential=toroidal)
        return out
    zc = np.zeros(ncoef, dtype=np.complex128)
    static_disp, static_grav, static_tan = zc.copy(), zc.copy(), zc.copy()
    if nz(displacement_response):
        static_disp += displacement_response
    if nz(potential_response):
        static_grav += potential_response
    if nz(tangential_response):
        static_tan += tangential_response
    load0 = {"u": 0.0, "phi": 0.0}
    numbers = channel_numbers or {}
    for key, field, first in (("u", displacement_load, 0), ("phi", potential_load, 0), ("v", tangential_traction, 1)):
        if not nz(field):
            continue
        lm = expand(field)
        h_c, k_c = np.array(numbers["h_" + key], float), np.array(numbers["k_" + key], float)
        l_c = np.array(numbers["l_" + key], float)
        l_c[0] = 0.0
        h_c[:first] = k_c[:first] = l_c[:first] = 0.0
        static_disp += h_c[degree] * lm
        static_grav += k_c[degree] * lm
        static_tan += l_c[degree] * lm
        if key in load0:
            load0[key] = lm[0].real
    if nz(tide):  # :533-545
        lt_t = np.zeros(lmax + 1) if lt_tide is None else np.array(lt_tide, dtype=np.float64)
        ht_, kt_ = np.array(ht, dtype=np.float64), np.array(kt, dtype=np.float64)
        ht_[0] = kt_[0] = lt_t[0] = 0.0
        static_disp += ht_[degree] * tide
        static_grav += kt_[degree] * tide
        static_tan += lt_t[degree] * tide
    static_slc = -(static_disp + static_grav / g)  # :590-600
    if nz(tide):
        static_slc -= tide / g
    if nz(solid_surface_change):
        static_slc -= expand(solid_surface_change)
    surface = lambda f: radius * radius * integrate(f)  # IntegrateSurface
    ocean_area = surface(ocean)
    per_area = 1.0 / ocean_area if ocean_area > 0.0 else 0.0  # InverseOceanArea
    direct = np.zeros(size)
    mean_slc = 0.0
    if direct_load is not None:
        direct = direct_load.copy()
        mean_slc = -surface(direct_load) * per_area / water_density
    if direct_load_outside is not None:
        direct = direct + direct_load_outside
    slc_factor = -(h + k / g)
    load_lm = expand(direct + water_density * ocean * mean_slc)
    rot = None
    if rotation:
        rot = _RotationFactors(rotation, h, k, np.asarray(ht), np.asarray(kt), radius, omega, polar, equatorial, G,
                               hc, kc, m_u, m_phi, m_c)
        static_disp2, static_grav2 = _block_of(static_disp), _block_of(static_grav)
        tide2 = _block_of(tide) if nz(tide) else np.zeros((2, 2))
        layer2 = _block_of(expand(solid_surface_change)) if nz(solid_surface_change) else np.zeros((2, 2))
        rotate = lambda lm: _rotation(rot, _block_of(lm), lm[0].real, static_disp2, static_grav2,
                                      inertia_moment_change, angular_momentum_change, load0["u"], load0["phi"])
    omega_out = np.zeros(3)
    mixer = AndersonMixer(anderson_memory)
    prev = None
    slc = np.zeros(size)
    err = np.inf
    converged = False
    count = 0
    shift = 0.0
    while count < max_iterations:
        lm = slc_factor[degree] * load_lm
        if any_static:
            lm = lm + static_slc
        if rot is not None:  # :625-640
            r = rotate(load_lm)
            omega_out = r["omega"]
            _set_block(lm, -(r["disp2"] + (r["grav2"] + r["centrifugal"] + tide2) / g + layer2))
            lm[0] -= (rot.hc + (rot.kc + 1.0) / g) * r["centrifugal0"]
        slc = synthesise(lm)
        shift = mean_slc - surface(ocean * slc) * per_area
        slc = slc + shift
        ocean_slc = ocean * slc
        if prev is not None:
            scale = np.max(np.abs(ocean_slc))
            err = np.max(np.abs(ocean_slc - prev)) / scale if scale > 0.0 else 0.0
            if err <= rtol:
                converged = True
                break
        prev = ocean_slc
        new_lm = expand(direct + water_density * prev)
        mixed = mixer.update(load_lm.view(np.float64), new_lm.view(np.float64))
        load_lm = mixed.view(np.complex128)
        count += 1
    tan = np.zeros(lmax + 1) if lt is None else np.array(lt, dtype=np.float64)
    tan[0] = 0.0
    disp_lm = h[degree] * load_lm + static_disp
    pot_lm = k[degree] * load_lm + static_grav
    tan_lm = tan[degree] * load_lm + static_tan
    if rot is not None:  # :714-724
        r = rotate(load_lm)
        _set_block(disp_lm, r["disp2"])
        _set_block(pot_lm, r["grav2"])
        disp_lm[0] += rot.hc * r["centrifugal0"]
        pot_lm[0] += rot.kc * r["centrifugal0"]
        lt2 = 0.0 if lt_tide is None else lt_tide[2]
        _add_block(tan_lm, lt2 * r["centrifugal"])
    out.update(sea_level_change=slc, displacement=synthesise(disp_lm), potential=synthesise(pot_lm),
               tangential_potential=synthesise(tan_lm), toroidal_potential=toroidal, uniform_shift=shift,
               iterations=count, error=err, converged=converged, angular_velocity=omega_out)
    return out


def flotation(ice, sea_level, water_density, ice_density, forced_land=None):
    """GRDSolver::MakeState's ocean function (src/SeaLevel.cpp:279-300):
    1 where the water column floats the ice (rho_w SL - rho_i I > 0) and the
    point is not held as land, else 0."""
    floats = water_density * np.asarray(sea_level) - ice_density * np.asarray(ice) > 0.0
    if forced_land is not None:
        floats &= np.asarray(forced_land) == 0
    return floats.astype(np.float64)


def solve_nonlinear(synthesise, expand, integrate, h, k, l, g, water_density, ice_density, radius, state,
                    ice_change=None, direct_load=None, direct_load_outside=None, solid_surface_change=None,
                    dynamic_sea_level_change=None, displacement_response=None, potential_response=None,
                    tangential_response=None, toroidal_response=None, tide=None, ht=None, kt=None, lt_tide=None,
                    rotation=0, omega=0.0, polar=0.0, equatorial=0.0, G=0.0, hc=0.0, kc=0.0, m_u=0.0, m_phi=0.0,
                    m_c=0.0, inertia_moment_change=0.0, forced_land="state", rtol=1e-9, max_iterations=50):
    """GRDSolver::SolveNonlinear (src/SeaLevel.cpp:970-1289): the sea level
    equation with migrating shorelines, a plain fixed point from the state
    given. `state` = dict(ice, sea_level, ocean, forced_land) (fields; the
    mask may be None). Each iteration: the total load of the current ocean
    function and sea level change (the grounded ice's and the water's
    changes from the state, formed from the changes, :1098-1110, and the
    direct loads), expanded; the sea level change of the load
    (-(h + k / g), the static terms and the rotation block); the water
    budget closed by a uniform shift over the current ocean (:1163-1180);
    then the new ocean function by flotation. Stops when the largest change
    of the sea level change between iterates is within rtol of its size,
    taken before and after the shift (:1196-1208). forced_land: "state" for
    the state's mask, else the mask held at this solve (None: none)."""
    h = np.asarray(h, dtype=np.float64)
    k = np.asarray(k, dtype=np.float64)
    lmax = h.size - 1
    degree = np.concatenate([np.full(m + 1, m) for m in range(lmax + 1)])
    ice0 = np.asarray(state["ice"], dtype=np.float64)
    bathy0 = np.asarray(state["sea_level"], dtype=np.float64)
    ocean0 = np.asarray(state["ocean"], dtype=np.float64)
    held = state.get("forced_land") if isinstance(forced_land, str) else forced_land
    size = ocean0.size
    surface = lambda f: radius * radius * integrate(f)  # IntegrateSurface
    if not surface(ocean0) > 0.0:
        raise ValueError("the nonlinear sea level solve needs a state with an ocean")
    tidal = tide is not None and np.max(np.abs(tide)) > 0.0
    static_disp = static_grav = static_slc = None
    if displacement_response is not None or potential_response is not None or tidal:
        static_disp = np.zeros(degree.size, dtype=np.complex128)
        static_grav = np.zeros(degree.size, dtype=np.complex128)
        if displacement_response is not None:
            static_disp = np.array(displacement_response, dtype=np.complex128)
        if potential_response is not None:
            static_grav = np.array(potential_response, dtype=np.complex128)
        if tidal:
            ht_, kt_ = np.array(ht, dtype=np.float64), np.array(kt, dtype=np.float64)
            ht_[0] = kt_[0] = 0.0
            static_disp = static_disp + ht_[degree] * tide
            static_grav = static_grav + kt_[degree] * tide
        static_slc = -(static_disp + static_grav / g)
        if tidal:
            static_slc = static_slc - tide / g
    layer2 = np.zeros((2, 2))
    if solid_surface_change is not None:
        layer_lm = expand(solid_surface_change)
        if static_slc is None:
            static_slc = np.zeros(degree.size, dtype=np.complex128)
        static_slc = static_slc - layer_lm
        layer2 = _block_of(layer_lm)
    tide2 = _block_of(tide) if tidal else np.zeros((2, 2))
    dice = np.zeros(size) if ice_change is None else np.asarray(ice_change, dtype=np.float64)
    new_ice = ice0 + dice
    direct = None
    direct_mass = 0.0
    if direct_load is not None:
        direct = np.array(direct_load, dtype=np.float64)
        direct_mass = surface(direct)
    if direct_load_outside is not None:
        direct = (np.zeros(size) if direct is None else direct) + direct_load_outside
    grounded = lambda c: ice_density * ((1.0 - c) * dice - (c - ocean0) * ice0)
    water = lambda c, change: water_density * (c * change + (c - ocean0) * bathy0)
    slc_factor = -(h + k / g)
    rot = None
    if rotation:
        rot = _RotationFactors(rotation, h, k, np.asarray(ht), np.asarray(kt), radius, omega, polar, equatorial, G,
                               hc, kc, m_u, m_phi, m_c)
        sd2 = _block_of(static_disp) if static_disp is not None else np.zeros((2, 2))
        sg2 = _block_of(static_grav) if static_grav is not None else np.zeros((2, 2))
        rotate = lambda lm: _rotation(rot, _block_of(lm), lm[0].real, sd2, sg2, inertia_moment_change, (0.0, 0.0, 0.0))
    ocean = ocean0.copy()
    change = np.zeros(size)
    slc_data = np.zeros(size)
    omega_out = np.zeros(3)
    last = None
    shift = 0.0
    err = np.inf
    converged = False
    count = 0
    load_lm = np.zeros(degree.size, dtype=np.complex128)
    while count < max_iterations:
        total = grounded(ocean) + water(ocean, change)
        if direct is not None:
            total = total + direct
        load_lm = expand(total)
        slc_lm = slc_factor[degree] * load_lm
        if static_slc is not None:
            slc_lm = slc_lm + static_slc
        if rot is not None:
            last = rotate(load_lm)
            omega_out = last["omega"]
            _set_block(slc_lm, -(last["disp2"] + (last["grav2"] + last["centrifugal"] + tide2) / g + layer2))
            slc_lm[0] -= (rot.hc + (rot.kc + 1.0) / g) * last["centrifugal0"]
        local = synthesise(slc_lm)
        raw = local if dynamic_sea_level_change is None else local + dynamic_sea_level_change
        unbalanced = grounded(ocean) + water(ocean, raw)
        shift = -(surface(unbalanced) + direct_mass) / (water_density * surface(ocean))
        new_slc = local + shift
        new_change = raw + shift
        floats = water_density * (bathy0 + new_change) - ice_density * new_ice > 0.0
        if held is not None:
            floats &= np.asarray(held) == 0
        top = max(np.max(np.abs(slc_data)), np.max(np.abs(local)) if count > 0 else 0.0)
        if top > 0.0:
            err = np.max(np.abs(new_slc - slc_data)) / top
        else:
            err = 0.0 if np.max(np.abs(new_slc)) == 0.0 else 1.0
        slc_data, change, ocean = new_slc, new_change, floats.astype(np.float64)
        count += 1
        if err <= rtol:
            converged = True
            break
    tan = np.zeros(lmax + 1) if l is None else np.array(l, dtype=np.float64)
    tan[0] = 0.0
    disp_lm = h[degree] * load_lm
    pot_lm = k[degree] * load_lm
    if static_disp is not None:
        disp_lm = disp_lm + static_disp
        pot_lm = pot_lm + static_grav
    tan_lm = tan[degree] * load_lm
    if tangential_response is not None:
        tan_lm = tan_lm + tangential_response
    if tidal:
        lt_t = np.zeros(lmax + 1) if lt_tide is None else np.array(lt_tide, dtype=np.float64)
        lt_t[0] = 0.0
        tan_lm = tan_lm + lt_t[degree] * tide
    if rot is not None and last is not None:
        _set_block(disp_lm, last["disp2"])
        _set_block(pot_lm, last["grav2"])
        disp_lm[0] += rot.hc * last["centrifugal0"]
        pot_lm[0] += rot.kc * last["centrifugal0"]
        lt2 = 0.0 if lt_tide is None else lt_tide[2]
        _add_block(tan_lm, lt2 * last["centrifugal"])
    carried = grounded(ocean) + water(ocean, change)
    if direct is not None:
        carried = carried + direct
    return dict(sea_level_change=slc_data, displacement=synthesise(disp_lm), potential=synthesise(pot_lm),
                tangential_potential=synthesise(tan_lm),
                toroidal_potential=synthesise(toroidal_response) if toroidal_response is not None else None,
                angular_velocity=omega_out, uniform_shift=shift, iterations=count, error=err, converged=converged,
                ice=new_ice, sea_level=bathy0 + change, ocean=ocean, ocean_area=surface(ocean),
                load_coefficients=expand(carried))

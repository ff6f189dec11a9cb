"""Input generators for the benchmark configurations, in chiML's JSON schema.

Each function returns a dict ready for ``write_json``; lengths are in units of
``a`` (100 nm), time in a/c, following the input conventions of chiML's reader
(INPUTS/parallelInputs.cpp). Random geometry is drawn from a seeded PCG64
generator (seed 20261203 + config id) so every run sees the same objects.
``scale`` shrinks a configuration for parity tests (fewer cells, same physics).
"""
import json
import math

import numpy as np

A = 1e-7                 # length unit (m)
C0 = 2.9979245e8         # speed of light, as the reference defines it
T_UNIT = A / C0          # one time unit in seconds
SEED0 = 20261203
C4_COUPLING = 1.0e2      # emitter coupling of the batched sweep (chiML's "couplings" units)
C4_AMPLITUDE = 5.0e8     # peak source amplitude of the batched sweep


def ev2fdtd(ev):
    """Photon energy in eV -> frequency in c/a (parallelInputs.cpp:1182-1185)."""
    return ev / 4.135666e-15 * A / C0


def _tlim(steps, dt):
    # ceil(tLim / dt) == steps for any rounding of the quotient
    return (steps - 0.5) * dt


def _obj(shape, loc, **kw):
    o = {"shape": shape, "loc": list(loc), "unit_vectors": [], "Basis_Set": []}
    o.update(kw)
    return o


def _gauss(fcen, fwidth, cutoff, t0, amp=1.0):
    return {"profile": "gaussian", "Field_Intensity": amp, "fcen": fcen, "fwidth": fwidth, "cutoff": cutoff, "t_0": t0}


def drude_lorentz_pols(wp_ev, poles):
    """Custom-material poles from (strength, width_eV, centre_eV) triples; centre 0 = Drude.

    Mirrors getMetal (parallelInputs.cpp:1187-1221): sigma = f (wp / Omega)^2 with
    Omega = 1e-20 eV for a Drude term; the JSON gamma / omega are the FDTD-unit
    values that the reader multiplies by pi and 2 pi.
    """
    wp = ev2fdtd(wp_ev)
    out = []
    for f, width_ev, centre_ev in poles:
        om = ev2fdtd(centre_ev if centre_ev != 0.0 else 1.0e-20)
        out.append({"gamma": ev2fdtd(width_ev), "omega": om, "sigma_p": f * (wp / om) ** 2})
    return out


def emitter_level(e_cen_ev, dist="Delta_Fxn", nstates=1, width_ev=None, levs=1):
    """One Energy_Levels entry (parallelInputs.cpp:465-579): centre in eV, optional
    broadening (a distribution sampled at nstates equispaced energies over +-2 widths)."""
    d = {"E_cen": [e_cen_ev], "distribution": dist, "nstates": nstates, "levs_described": levs}
    if width_ev is not None:
        d["dist_width"] = [width_ev]
        d["BandWith"] = 4.0 * width_ev
    return d


def emitter_obj(shape, loc, basis, levels, couplings, relax, mol_den, eps=1.0, dtc_levs=(), output_pol=None,
                dtc_base="out/qe_", **geo):
    """An object holding quantum emitters (parallelInputs.cpp:425-662): (l, m) basis,
    energy levels, coupling matrix, relaxation channels (state_i, state_f, rate 1/s,
    dephasing rate 1/s), molecular density (1/m^3), population detectors and the
    polarisation output file."""
    o = _obj(shape, loc, material="custom", eps=eps, pols=[], **geo)
    o["Basis_Set"] = [{"l": l, "m": m} for (l, m) in basis]
    o["mol_den"] = mol_den
    o["Energy_Levels"] = list(levels)
    o["couplings"] = [float(c) for c in couplings]
    o["gam"] = []
    o["RelaxationOperators"] = [{"state_i": i, "state_f": f, "rate": r, "dephasing_rate": d} for (i, f, r, d) in relax]
    o["dtc_levs"] = list(dtc_levs)
    o["levDTC_timeInt"] = 1
    o["dtc_pop_fname_base"] = dtc_base
    if output_pol:
        o["output_pol"] = True
        o["output_pol_filename"] = output_pol
    return o


def config1(n=400, pml=20, steps=4000, radius_cells=50, src_gap_cells=60, ndtc=8, nfreq=100):
    """2-D TMz (Ez, Hx, Hy), dielectric disk eps=2.25, Ez point source, 8 point detectors, flux line."""
    dx = 0.05
    dt = dx / 2.0
    size = (n - 1) * dx
    r = radius_cells * dx
    width = 2e-15 / T_UNIT
    t0 = 6e-15 / T_UNIT
    src_x = -(r + src_gap_cells * dx)
    dets = []
    for k in range(ndtc):
        ang = 2 * math.pi * k / ndtc
        rr = r + 0.35 * (size / 2 - pml * dx - r)
        p = [round(rr * math.cos(ang) / dx) * dx, round(rr * math.sin(ang) / dx) * dx, 0.0]
        dets.append({"loc": p, "size": [0.0, 0.0, 0.0], "type": "Ez", "fname": "out/c1_pt%d" % k,
                     "dtc_class": "txt", "SI": False, "Time_Interval": dt})
    flux_x = round((size / 2 - pml * dx - 4 * dx) / dx) * dx
    flux_h = round((size - 2 * pml * dx - 10 * dx) / dx) * dx
    return {
        "CompCell": {"size": [size, size, 0.0], "stepSize": [dx, dx, dx], "dt": dt, "tLim": _tlim(steps, dt),
                     "a": A, "pol": "Ez", "PBC": False, "InputMaps_x": [], "InputMaps_y": [], "InputMaps_z": []},
        "PML": {"thickness": [pml * dx, pml * dx, 0.0], "m": 3.0, "ma": 1.0, "sigOptRat": 1.0, "kappaMax": 1.0, "aMax": 0.0},
        "SourceList": [{"pol": "Ez", "loc": [round(src_x / dx) * dx, 0.0, 0.0], "size": [0.0, 0.0, 0.0],
                        "PulseList": [_gauss(A / 500e-9, 1.0 / width, 5.0, t0)]}],
        "TFSF": [],
        "ObjectList": [_obj("sphere", [0.0, 0.0, 0.0], radius=r, material="custom", eps=2.25, pols=[])],
        "DetectorList": dets,
        "FluxList": [{"name": "out/c1_flux", "loc": [flux_x, 0.0, 0.0], "size": [0.0, flux_h, 0.0],
                      "lamL": 4.0, "lamR": 7.0, "nfreq": nfreq, "SI": False}],
    }


def tfsf_surface(box, fcen_a, width, psi_deg=0.0, theta_deg=0.0, phi_deg=90.0, m=None, circ=None, pml_thick=12,
                 loc=(0.0, 0.0, 0.0), amp=1.0):
    """One TFSF entry (parallelInputs.cpp:219-408): box size (a units), a Gaussian pulse at
    fcen_a (1/a units) of 1/e time width ``width``, direction from theta/phi or an integer
    vector m, polarisation angle psi (0 = along x for propagation along z), optional
    circular polarisation ("L" / "R"), the thickness of its 1-D CPML and the peak amplitude."""
    t = {"loc": list(loc), "size": list(box), "theta": theta_deg, "phi": phi_deg, "psi": psi_deg,
         "PulseList": [_gauss(fcen_a, 1.0 / width, 4.0, 3 * width, amp=amp)], "pmlThick": pml_thick}
    if m is not None:
        t["m"] = list(m)
    if circ:
        t["circPol"] = circ
    return t


def config2(n=256, pml=12, steps=5000, nell=16, nfreq=150, seed=SEED0 + 2, metal_radius_cells=30, aniso=True,
            tfsf=True):
    """3-D dispersive scene: seeded ellipsoids, a Drude + 2 Lorentz metal sphere, an
    x-polarised plane wave along +z and a DFT flux box. With ``tfsf`` the wave enters
    through a TFSF box (4 cells inside the CPML) that holds every object and the flux box;
    without it, through a soft Ex source sheet.

    With ``aniso`` each ellipsoid is uniaxial: eps_inf = eps_o plus one oriented-dipole
    Lorentz pole along the random optic axis whose static strength is eps_e - eps_o, centred
    far above the source band (5x its centre frequency), so that the permittivity along the
    axis is eps_e and across it eps_o. The pair (eps_o, eps_e) is drawn as two uniforms on
    [1.5, 4] ordered so that eps_e >= eps_o (the reader drops the direction of a pole with
    negative strength)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = 0.05
    dt = 0.5 * dx / math.sqrt(3.0)
    size = (n - 1) * dx
    half = size / 2
    inner = half - (pml + 6) * dx
    objs = []
    for _ in range(nell):
        semi = rng.uniform(10, 40, size=3) * dx * (n / 256.0)
        e1 = float(rng.uniform(1.5, 4.0))
        e2 = float(rng.uniform(1.5, 4.0))
        eps_o, eps_e = (min(e1, e2), max(e1, e2)) if aniso else (e1, e1)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        lim = np.maximum(inner - semi.max(), 0.0)
        c = rng.uniform(-lim, lim, size=3)
        u0 = axis
        tmp = np.array([1.0, 0.0, 0.0]) if abs(axis[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        u1 = np.cross(u0, tmp)
        u1 /= np.linalg.norm(u1)
        u2 = np.cross(u0, u1)
        pols = []
        if aniso and eps_e > eps_o:
            pols = [{"gamma": 0.01, "omega": 5.0 * A / 550e-9, "sigma_p": eps_e - eps_o,
                     "dipOrE": "unidirectional", "dirDipE": [float(v) for v in axis]}]
        objs.append(_obj("ellipsoid", [float(v) for v in c], size=[float(2 * s) for s in semi], material="custom",
                         eps=eps_o, pols=pols,
                         unit_vectors=[{"uvec": [float(v) for v in u]} for u in (u0, u1, u2)]))
    rm = metal_radius_cells * dx * (n / 256.0)
    objs.append(_obj("sphere", [0.0, 0.0, 0.0], radius=rm, material="custom", eps=6.0,
                     pols=drude_lorentz_pols(9.0, [(1.0, 0.07, 0.0), (1.0, 0.4, 2.6), (0.5, 0.8, 3.5)])))
    src_z = -(half - (pml + 3) * dx)
    sheet = size - 2 * (pml + 1) * dx
    fb = 2 * (half - (pml + 5) * dx)
    width = 5e-15 / T_UNIT
    tbox = 2 * (half - (pml + 4) * dx)
    tf = [tfsf_surface([tbox] * 3, A / 550e-9, width, psi_deg=0.0, theta_deg=0.0)] if tfsf else []
    srcs = [] if tfsf else [{"pol": "Ex", "loc": [0.0, 0.0, round(src_z / dx) * dx], "size": [sheet, sheet, 0.0],
                             "PulseList": [_gauss(A / 550e-9, 1.0 / width, 4.0, 3 * width)]}]
    return {
        "CompCell": {"size": [size, size, size], "stepSize": [dx, dx, dx], "dt": dt, "tLim": _tlim(steps, dt),
                     "a": A, "pol": "Ex", "PBC": False, "InputMaps_x": [], "InputMaps_y": [], "InputMaps_z": []},
        "PML": {"thickness": [pml * dx] * 3, "m": 3.0, "ma": 1.0, "sigOptRat": 1.0, "kappaMax": 1.0, "aMax": 0.0},
        "SourceList": srcs,
        "TFSF": tf,
        "ObjectList": objs,
        "DetectorList": [{"loc": [0.0, 0.0, round((half - (pml + 8) * dx) / dx) * dx], "size": [0.0, 0.0, 0.0],
                          "type": "Ex", "fname": "out/c2_pt", "dtc_class": "txt", "SI": False, "Time_Interval": dt}],
        "FluxList": [{"name": "out/c2_flux", "loc": [0.0, 0.0, 0.0], "size": [fb, fb, fb],
                      "lamL": 4.0, "lamR": 7.0, "nfreq": nfreq, "SI": False}],
    }


def config3(n=192, pml=12, steps=8000, slab_cells=20, nstates=3, mol_den=1e26, coupling=C4_COUPLING, nfreq=50,
            cell_dipoles=True, seed=SEED0 + 3):
    """3-D Maxwell-Liouville scene: a ``slab_cells``-thick slab (normal z) of three-level
    ladder emitters across the cell inside the CPML, transitions at 2.0 and 2.2 eV with
    Gaussian inhomogeneous broadening of 20 meV sampled at ``nstates`` energies per upper
    level (nstates^2 ensemble members per cell), T1 = 1 ps and T2 = 50 fs on both
    transitions, ground-state start; an Ez plane source sheet below the slab with a
    Gaussian pulse at 2.1 eV, 10 fs wide, peak 5e8 V/m; a flux plane above
    the slab, a point detector and the upper-level populations. With ``cell_dipoles`` each
    cell's dipole points in its own seeded random direction (the per-cell dipole extension:
    ``dipole_orientation``), otherwise along z as in the reference."""
    dx = 0.05
    dt = 0.5 * dx / math.sqrt(3.0)
    size = (n - 1) * dx
    half = size / 2
    inner = size - 2 * (pml + 2) * dx
    lv = [emitter_level(0.0), emitter_level(2.0, "Gaussian", nstates, 0.02), emitter_level(4.2, "Gaussian", nstates, 0.02)]
    relax = [(1, 0, 1e12, 1.0 / 50e-15), (2, 1, 1e12, 1.0 / 50e-15)]
    qe = emitter_obj("block", [0.0, 0.0, 0.0], [(0, 0), (1, 0), (2, 0)], lv, [coupling] * 9, relax, mol_den, eps=1.0,
                     dtc_levs=[0, 4, 8], output_pol="c3_pol.dat", dtc_base="c3_qe_",
                     size=[inner, inner, slab_cells * dx])
    if cell_dipoles:
        qe.update(dipole_orientation="random", dipole_seed=seed)
    width = 10e-15 / T_UNIT
    src_z = -round((half - (pml + 4) * dx) / dx) * dx
    out_z = round((half - (pml + 6) * dx) / dx) * dx
    return {
        "CompCell": {"size": [size, size, size], "stepSize": [dx, dx, dx], "dt": dt, "tLim": _tlim(steps, dt),
                     "a": A, "pol": "Ez", "PBC": False, "InputMaps_x": [], "InputMaps_y": [], "InputMaps_z": []},
        "PML": {"thickness": [pml * dx] * 3, "m": 3.0, "ma": 1.0, "sigOptRat": 1.0, "kappaMax": 1.0, "aMax": 0.0},
        "SourceList": [{"pol": "Ez", "loc": [0.0, 0.0, src_z], "size": [inner, inner, 0.0],
                        "PulseList": [_gauss(ev2fdtd(2.1), 1.0 / width, 4.0, 3 * width, amp=C4_AMPLITUDE)]}],
        "TFSF": [],
        "ObjectList": [qe],
        "DetectorList": [{"loc": [0.0, 0.0, out_z], "size": [0.0, 0.0, 0.0], "type": "Ez", "fname": "c3_pt",
                          "dtc_class": "txt", "SI": False, "Time_Interval": dt}],
        "FluxList": [{"name": "c3_flux", "loc": [0.0, 0.0, out_z], "size": [inner, inner, 0.0],
                      "lamL": 5.0, "lamR": 7.0, "nfreq": nfreq, "SI": False}],
    }


def config5(n=640, nz=320, pml=16, steps=20000, nell=16, nfreq=200, seed=SEED0 + 5, coupling=C4_COUPLING,
            mol_den=1e26, sheet_cells=10, film_cells=10, amp=C4_AMPLITUDE, cell_dipoles=True):
    """Large 3-D mixed scene (dx = 4 nm, fields in FP32 in the split form): n x n x nz cells.

    Inside the total-field box of a TFSF surface (``pml`` + 4 cells in from the edges): a
    ``film_cells``-thick Drude metal film (wp = 9 eV, gamma = 0.07 eV) below the middle, a
    ``sheet_cells``-thick sheet of four-level ladder emitters above it (transitions at 1.9,
    2.0 and 2.3 eV, FP64 density matrices; with ``cell_dipoles`` every cell's dipole points in
    its own seeded random direction with a magnitude drawn from 0.5-1.5 x ``coupling`` (the
    5-15 D dipoles of the configuration, through the per-cell dipole extension), otherwise
    z dipoles whose adjacent-level couplings are drawn from 0.5-1.5 x ``coupling`` (a
    stand-in the reference can run: it has one
    dipole operator per emitter object, so the draw is per transition, not per cell), and
    ``nell`` seeded uniaxial ellipsoids between the two, built as in config 2. The wave is a
    p-polarised Gaussian pulse at 550 nm along m = (1, 1, 3) (25 degrees off the film
    normal, so its E field has a z component that drives the emitters), peak ``amp``. Six
    DFT flux planes of ``nfreq`` frequencies, three below the film and three above the
    sheet."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dx = 0.04
    dt = 0.5 * dx / math.sqrt(3.0)
    sx = (n - 1) * dx
    sz = (nz - 1) * dx
    hx, hz = sx / 2, sz / 2
    box_x = hx - (pml + 4) * dx           # half sizes of the TFSF box
    box_z = hz - (pml + 4) * dx
    cell = lambda v: round(v / dx) * dx
    film_z = cell(-0.55 * box_z)
    sheet_z = cell(0.55 * box_z)
    lateral = 2 * (hx - (pml + 12) * dx)
    inner_x = hx - (pml + 6) * dx
    room_z = 0.55 * box_z - 0.5 * max(film_cells, sheet_cells) * dx - dx
    objs = []
    for _ in range(nell):
        semi = rng.uniform(10, 40, size=3) * dx * (n / 640.0)
        e1, e2 = float(rng.uniform(1.5, 4.0)), float(rng.uniform(1.5, 4.0))
        eps_o, eps_e = min(e1, e2), max(e1, e2)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        lim = np.maximum(np.array([inner_x, inner_x, room_z]) - semi.max(), 0.0)
        c = rng.uniform(-lim, lim)
        tmp = np.array([1.0, 0.0, 0.0]) if abs(axis[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        u1 = np.cross(axis, tmp)
        u1 /= np.linalg.norm(u1)
        u2 = np.cross(axis, u1)
        pols = [{"gamma": 0.01, "omega": 5.0 * A / 550e-9, "sigma_p": eps_e - eps_o, "dipOrE": "unidirectional",
                 "dirDipE": [float(v) for v in axis]}] if eps_e > eps_o else []
        objs.append(_obj("ellipsoid", [float(v) for v in c], size=[float(2 * s) for s in semi], material="custom",
                         eps=eps_o, pols=pols, unit_vectors=[{"uvec": [float(v) for v in u]} for u in (axis, u1, u2)]))
    objs.append(_obj("block", [0.0, 0.0, film_z], size=[lateral, lateral, film_cells * dx], material="custom",
                     eps=1.0, pols=drude_lorentz_pols(9.0, [(1.0, 0.07, 0.0)])))
    nlev = 4
    cpl = np.zeros((nlev, nlev))
    for a in range(nlev - 1):
        draw = float(rng.uniform(0.5, 1.5))
        cpl[a, a + 1] = cpl[a + 1, a] = coupling * (1.0 if cell_dipoles else draw)
    lv = [emitter_level(0.0), emitter_level(1.9), emitter_level(3.9), emitter_level(6.2)]
    relax = [(1, 0, 1e12, 2e13), (2, 1, 1e12, 2e13), (3, 2, 1e12, 2e13)]
    objs.append(emitter_obj("block", [0.0, 0.0, sheet_z], [(0, 0), (1, 0), (2, 0), (3, 0)], lv,
                            [float(v) for v in cpl.ravel()], relax, mol_den, eps=1.0, dtc_levs=[5, 10, 15],
                            output_pol="c5_pol.dat", dtc_base="c5_qe_", size=[lateral, lateral, sheet_cells * dx]))
    if cell_dipoles:
        objs[-1].update(dipole_orientation="random", dipole_seed=seed, dipole_scale_range=[0.5, 1.5])
    width = 5e-15 / T_UNIT
    fl = 2 * (hx - (pml + 6) * dx)
    planes = []
    for k, zf in enumerate((-0.94, -0.87, -0.8, 0.8, 0.87, 0.94)):
        planes.append({"name": "c5_flux%d" % k, "loc": [0.0, 0.0, cell(zf * box_z)], "size": [fl, fl, 0.0],
                       "lamL": 4.0, "lamR": 7.0, "nfreq": nfreq, "SI": False})
    tf = tfsf_surface([2 * box_x, 2 * box_x, 2 * box_z], A / 550e-9, width, psi_deg=90.0, m=(1, 1, 3),
                      pml_thick=pml, amp=amp)
    return {
        "CompCell": {"size": [sx, sx, sz], "stepSize": [dx, dx, dx], "dt": dt, "tLim": _tlim(steps, dt),
                     "a": A, "pol": "Ex", "PBC": False, "InputMaps_x": [], "InputMaps_y": [], "InputMaps_z": []},
        "PML": {"thickness": [pml * dx] * 3, "m": 3.0, "ma": 1.0, "sigOptRat": 1.0, "kappaMax": 1.0, "aMax": 0.0},
        "SourceList": [],
        "TFSF": [tf],
        "ObjectList": objs,
        "DetectorList": [],
        "FluxList": planes,
    }


def config4_member(side, detuning_ev, mol_den, pml=16, steps=6000, sheet_cells=10, coupling=C4_COUPLING,
                   nfreq=50, tag="c4"):
    """One point of the batched sweep: a 2-D TMz square of ``side`` cells (dx = 5 nm) with a
    ``sheet_cells``-thick sheet of two-level emitters (z dipoles) across the whole width,
    transition at 2.0 eV + ``detuning_ev``, dephasing T2 = 30 fs and population decay
    T1 = 1 ps; an Ez line source on one side, a point detector and a DFT flux line on the
    other, and the upper-level population recorded every step."""
    dx = 0.05
    dt = dx / 2.0
    size = (side - 1) * dx
    half = size / 2
    e0 = 2.0
    width = 10e-15 / T_UNIT
    lv = [emitter_level(0.0), emitter_level(e0 + detuning_ev)]
    sheet_h = size - 2 * (pml + 2) * dx
    obj = emitter_obj("block", [0.0, 0.0, 0.0], [(0, 0), (1, 0)], lv, [coupling] * 4,
                      [(1, 0, 1e12, 1.0 / 30e-15)], mol_den, eps=1.0, dtc_levs=[3],
                      output_pol=tag + "_pol.dat", dtc_base=tag + "_qe_",
                      size=[sheet_cells * dx, sheet_h, 0.0])
    src_x = -round((half - (pml + 4) * dx) / dx) * dx
    out_x = round((half - (pml + 6) * dx) / dx) * dx
    return {
        "CompCell": {"size": [size, size, 0.0], "stepSize": [dx, dx, dx], "dt": dt, "tLim": _tlim(steps, dt),
                     "a": A, "pol": "Ez", "PBC": False, "InputMaps_x": [], "InputMaps_y": [], "InputMaps_z": []},
        "PML": {"thickness": [pml * dx, pml * dx, 0.0], "m": 3.0, "ma": 1.0, "sigOptRat": 1.0, "kappaMax": 1.0, "aMax": 0.0},
        "SourceList": [{"pol": "Ez", "loc": [src_x, 0.0, 0.0], "size": [0.0, sheet_h, 0.0],
                        "PulseList": [_gauss(ev2fdtd(e0), 1.0 / width, 4.0, 3 * width, amp=C4_AMPLITUDE)]}],
        "TFSF": [],
        "ObjectList": [obj],
        "DetectorList": [{"loc": [out_x, 0.0, 0.0], "size": [0.0, 0.0, 0.0], "type": "Ez", "fname": tag + "_pt",
                          "dtc_class": "txt", "SI": False, "Time_Interval": dt}],
        "FluxList": [{"name": tag + "_flux", "loc": [out_x, 0.0, 0.0], "size": [0.0, sheet_h, 0.0],
                      "lamL": 5.0, "lamR": 7.5, "nfreq": nfreq, "SI": False}],
    }


def config4(n=96, sides=tuple(range(192, 769, 64)), steps=6000, seed=SEED0 + 4, pml=16):
    """The batched sweep: ``n`` independent 2-D TMz emitter simulations. Square sides are
    drawn by seed from ``sides``; detuning runs over -100..+100 meV and molecular density
    over 1e25..1e26 m^-3 (log-spaced) on a grid of the two, in sweep order. Returns
    [(name, cfg)]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nd = max(1, int(round(math.sqrt(n * 1.5))))
    while n % nd:
        nd -= 1
    nn = n // nd
    dets = np.linspace(-0.1, 0.1, nd) if nd > 1 else np.zeros(1)
    dens = np.logspace(25, 26, nn) if nn > 1 else np.array([1e25])
    out = []
    for k in range(n):
        side = int(rng.choice(np.asarray(sides)))
        det, den = float(dets[k % nd]), float(dens[k // nd])
        name = "c4_%03d" % k
        out.append((name, config4_member(side, det, den, pml=pml, steps=steps, tag=name)))
    return out


def write_json(cfg, path):
    with open(path, "w") as f:
        json.dump(cfg, f, indent=1)
    return path

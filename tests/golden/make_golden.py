"""Regenerates the golden fixtures from the reference's own CPU build.

For every case in CASES this writes <case>/in.json (from chiml_gb300.configs),
runs the one-process build of the chiML sources (oracle/_ref/chiml_ref, made by
oracle/Makefile.ref) on it in a scratch directory, and copies every output file
it writes into <case>/ref/. Run it where the chiML sources are available:

    python tests/golden/make_golden.py
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from chiml_gb300 import configs  # noqa: E402


def _te_dispersive():
    """2-D TE (Ex, Ey, Hz): Drude-Lorentz disk, Ey point source, binary box detector, flux box."""
    cfg = configs.config1(n=72, pml=8, steps=260, radius_cells=9, src_gap_cells=10, ndtc=2, nfreq=9)
    cfg["CompCell"]["pol"] = "Hz"
    cfg["SourceList"][0]["pol"] = "Ey"
    cfg["ObjectList"] = [configs._obj("sphere", [0.0, 0.0, 0.0], radius=0.45, material="custom", eps=2.0,
                                      pols=configs.drude_lorentz_pols(4.0, [(1.0, 0.2, 0.0), (0.6, 0.3, 2.4)]))]
    for d in cfg["DetectorList"]:
        d["type"] = "Hz"
    cfg["DetectorList"].append({"loc": [0.5, 0.3, 0.0], "size": [0.2, 0.1, 0.0], "type": "Ey",
                                "fname": "out/te_box", "dtc_class": "bin", "SI": True, "Time_Interval": 2 * cfg["CompCell"]["dt"]})
    cfg["FluxList"] = [{"name": "out/te_flux", "loc": [0.0, 0.0, 0.0], "size": [1.6, 1.6, 0.0],
                        "lamL": 3.0, "lamR": 8.0, "nfreq": 9, "SI": True}]
    return cfg


def _tm_lorentz():
    """2-D TMz with a two-pole Lorentz disk and an E_pow box detector."""
    cfg = configs.config1(n=64, pml=8, steps=240, radius_cells=8, src_gap_cells=9, ndtc=3, nfreq=10)
    cfg["ObjectList"][0]["pols"] = configs.drude_lorentz_pols(6.0, [(0.5, 0.3, 2.0), (0.4, 0.5, 3.1)])
    cfg["ObjectList"][0]["eps"] = 1.5
    cfg["DetectorList"].append({"loc": [0.6, -0.2, 0.0], "size": [0.1, 0.15, 0.0], "type": "Ez",
                                "fname": "out/tm_box", "dtc_class": "bin", "SI": False, "Time_Interval": 3 * cfg["CompCell"]["dt"]})
    return cfg


def _qe_pulse(amp=5e8):
    return [configs._gauss(configs.ev2fdtd(2.0), 1.0 / (10e-15 / configs.T_UNIT), 5.0, 12e-15 / configs.T_UNIT, amp=amp)]


def _qe_tm():
    """2-D TMz with a block of two-level emitters (z dipoles), relaxation and dephasing."""
    cfg = configs.config1(n=60, pml=8, steps=300, radius_cells=6, src_gap_cells=6, ndtc=2, nfreq=4)
    lv = [configs.emitter_level(0.0), configs.emitter_level(2.0)]
    cfg["ObjectList"] = [configs.emitter_obj("block", [0.0, 0.0, 0.0], [(0, 0), (1, 0)], lv, [1e5] * 4,
                                             [(1, 0, 1e12, 2e13)], 1e21, eps=1.5, dtc_levs=[0, 3],
                                             output_pol="out/qe_pol.dat", size=[0.4, 0.4, 0.0])]
    cfg["SourceList"][0]["loc"] = [-0.3, 0.0, 0.0]
    cfg["SourceList"][0]["PulseList"] = _qe_pulse()
    return cfg


def _qe_te():
    """2-D TE (Ex, Ey, Hz) with a disk of emitters in an (l, m) = (0,0), (1,1), (1,-1) basis (x/y dipoles)."""
    cfg = configs.config1(n=56, pml=8, steps=260, radius_cells=6, src_gap_cells=6, ndtc=2, nfreq=4)
    cfg["CompCell"]["pol"] = "Hz"
    cfg["SourceList"][0]["pol"] = "Ey"
    cfg["SourceList"][0]["loc"] = [-0.6, 0.1, 0.0]
    cfg["SourceList"][0]["PulseList"] = _qe_pulse()
    for d in cfg["DetectorList"]:
        d["type"] = "Ex"
    lv = [configs.emitter_level(0.0), configs.emitter_level(2.0, levs=2)]
    cfg["ObjectList"] = [configs.emitter_obj("sphere", [0.0, 0.0, 0.0], [(0, 0), (1, 1), (1, -1)], lv, [1e5] * 9,
                                             [(1, 0, 1e12, 2e13), (2, 0, 1e12, 0.0)], 1e21, eps=1.3, dtc_levs=[0, 4, 8],
                                             output_pol="out/qe_te_pol.dat", radius=0.25)]
    cfg["FluxList"][0]["name"] = "out/qe_te_flux"
    return cfg


def _qe_3d():
    """3-D ladder of three levels (z dipoles) with Gaussian-broadened upper levels (nine ensemble
    members), Ez plane source, population detectors and the polarisation output."""
    n, dx = 26, 0.05
    cfg = configs.config2(n=n, pml=5, steps=90, nell=0, nfreq=4, metal_radius_cells=0, tfsf=False)
    cfg["ObjectList"] = []
    lv = [configs.emitter_level(0.0), configs.emitter_level(2.0, "Gaussian", 3, 0.02),
          configs.emitter_level(4.2, "Gaussian", 3, 0.02)]
    cfg["ObjectList"].append(configs.emitter_obj("block", [0.0, 0.0, 0.05], [(0, 0), (1, 0), (2, 0)], lv, [1e5] * 9,
                                                 [(1, 0, 1e12, 2e13), (2, 1, 1e12, 2e13)], 1e21, eps=1.2,
                                                 dtc_levs=[0, 4, 8], output_pol="out/qe3d_pol.dat",
                                                 size=[0.3, 0.3, 0.15]))
    src = cfg["SourceList"][0]
    src["pol"] = "Ez"
    src["PulseList"] = _qe_pulse()
    return cfg


def _c2_aniso():
    """3-D with five uniaxial ellipsoids (oriented-dipole poles) and the metal sphere; a short
    pulse so that the field reaches the objects within the run."""
    cfg = configs.config2(n=36, pml=6, steps=160, nell=5, nfreq=6, metal_radius_cells=18, tfsf=False)
    width = 0.3e-15 / configs.T_UNIT
    cfg["SourceList"][0]["PulseList"] = [configs._gauss(configs.A / 550e-9, 1.0 / width, 4.0, 2 * width)]
    return cfg


def _tfsf_disp():
    """3-D TFSF plane wave along +z, x-polarised, onto three uniaxial ellipsoids and the
    Drude-Lorentz sphere inside the total-field box; a short pulse that crosses the box."""
    cfg = configs.config2(n=40, pml=6, steps=240, nell=2, nfreq=6, metal_radius_cells=36, tfsf=True)
    width = 0.2e-15 / configs.T_UNIT
    cfg["TFSF"][0]["PulseList"] = [configs._gauss(configs.A / 550e-9, 1.0 / width, 4.0, 2 * width)]
    cfg["TFSF"][0]["pmlThick"] = 8
    return cfg


def _tfsf_oblique():
    """3-D oblique TFSF (m = (1, 2, 1)), left circular polarisation, onto a dispersive sphere."""
    cfg = configs.config2(n=32, pml=6, steps=160, nell=0, nfreq=5, metal_radius_cells=40, tfsf=True)
    dx = 0.05
    box = 2 * ((32 - 1) * dx / 2 - 10 * dx)
    width = 0.2e-15 / configs.T_UNIT
    cfg["TFSF"] = [configs.tfsf_surface([box] * 3, configs.A / 550e-9, width, psi_deg=20.0, m=(1, 2, 1), circ="L",
                                        pml_thick=6)]
    return cfg


def _tfsf_2d_te():
    """2-D TE (Ex, Ey, Hz) TFSF along m = (1, 1, 0) onto the dielectric disk, flux line inside."""
    cfg = configs.config1(n=60, pml=8, steps=240, radius_cells=6, src_gap_cells=6, ndtc=2, nfreq=5)
    cfg["CompCell"]["pol"] = "Hz"
    cfg["SourceList"] = []
    for d in cfg["DetectorList"]:
        d["type"] = "Ey"
    dx = 0.05
    box = 2 * ((60 - 1) * dx / 2 - 12 * dx)
    width = 0.3e-15 / configs.T_UNIT
    cfg["TFSF"] = [configs.tfsf_surface([box, box, 0.0], configs.A / 550e-9, width, m=(1, 1, 0), pml_thick=10)]
    return cfg


def _freq_dets(cfg, dets):
    """Appends frequency-domain detectors (type, size, output_map, SI, interval in steps) at the centre."""
    dt = cfg["CompCell"]["dt"]
    for i, (typ, sz, maps, si, ti) in enumerate(dets):
        cfg["DetectorList"].append({"loc": [0.0, 0.0, 0.0], "size": list(sz), "type": typ, "fname": "out/fq%d" % i,
                                    "dtc_class": "freq", "SI": si, "Time_Interval": ti * dt, "lamL": 4.0, "lamR": 7.0,
                                    "nfreq": 5, "output_map": maps})
    return cfg


def _freq_3d():
    """Frequency-domain detectors in 3-D under a TFSF plane wave: an Ex box in SI units, an E power
    box sampled every other step, an H power box written as per-frequency maps, an Hy plane."""
    return _freq_dets(_tfsf_disp(), [("Ex", (0.2, 0.2, 0.2), False, True, 1), ("E_pow", (0.1, 0.15, 0.2), False, False, 2),
                                     ("H_pow", (0.1, 0.1, 0.1), True, True, 1), ("Hy", (0.1, 0.0, 0.1), False, False, 3)])


def _freq_2d():
    """Frequency-domain detectors in 2-D TE (the reference's storage holds no points there:
    the field columns are zero, the incident columns are not)."""
    return _freq_dets(_tfsf_2d_te(), [("Ey", (0.2, 0.2, 0.0), False, False, 1), ("H_pow", (0.1, 0.1, 0.0), True, True, 1)])


def _c5_small():
    """Config 5 in miniature: three uniaxial ellipsoids, the Drude film, the four-level emitter
    sheet, the oblique p-polarised TFSF wave and the six flux planes, at 40 x 40 x 48 cells."""
    return configs.config5(n=40, nz=48, pml=6, steps=480, nell=3, nfreq=5, sheet_cells=2, film_cells=2, cell_dipoles=False)


def _bin_planes(cfg, planes, every=20):
    """Binary snapshot detectors of Ex over planes through the objects (box size, fname)."""
    dt = cfg["CompCell"]["dt"]
    for k, (typ, size) in enumerate(planes):
        cfg["DetectorList"].append({"loc": [0.0, 0.0, 0.0], "size": list(size), "type": typ, "fname": "out/plane%d" % k,
                                    "dtc_class": "bin", "SI": False, "Time_Interval": every * dt})
    return cfg


def _shape(shape, loc, eps, pols=None, **kw):
    return configs._obj(shape, loc, material="custom", eps=eps, pols=pols or [], **kw)


def _rot(theta_deg, phi_deg):
    """unit_vectors of a frame rotated by theta about y, then phi about z."""
    import math
    t, p = math.radians(theta_deg), math.radians(phi_deg)
    u0 = [math.cos(t) * math.cos(p), math.cos(t) * math.sin(p), -math.sin(t)]
    u1 = [-math.sin(p), math.cos(p), 0.0]
    u2 = [math.sin(t) * math.cos(p), math.sin(t) * math.sin(p), math.cos(t)]
    return [{"uvec": u} for u in (u0, u1, u2)]


def _shapes_a():
    """3-D: the cone (first, so the others overwrite it: the reference's cone test bounds it in
    y only), a hemisphere, a rotated hemiellipsoid, a rounded block, a partial torus and a
    paraboloid, one of them with a Lorentz pole; Ex plane source, flux box, two BIN planes."""
    cfg = configs.config2(n=44, pml=6, steps=200, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    lor = configs.drude_lorentz_pols(5.0, [(0.6, 0.3, 2.4)])
    cfg["ObjectList"] = [
        _shape("cone", [-0.4, 0.35, 0.0], 1.4, radSmall=0.05, radLarge=0.15, height=0.3),
        _shape("hemisphere", [-0.4, -0.3, 0.0], 2.0, radius=0.16, orPhi=30.0),
        _shape("hemiellipsoid", [0.0, -0.3, 0.05], 2.5, size=[0.3, 0.22, 0.26], unit_vectors=_rot(25.0, 40.0)),
        _shape("block", [0.4, -0.3, 0.0], 3.0, size=[0.3, 0.26, 0.22], rad_curve=0.06, unit_vectors=_rot(10.0, 15.0)),
        _shape("torus", [0.0, 0.3, 0.0], 2.2, pols=lor, rad_Ring=0.13, rad_CrossSec=0.06, phiMin=20.0, phiMax=290.0,
               unit_vectors=_rot(30.0, 0.0)),
        _shape("paraboloid", [0.4, 0.3, 0.0], 1.8, a=0.28, b=0.2, length=0.3, orTheta=60.0, orPhi=20.0),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Ey", (0.0, 1.5, 1.5))])


def _shapes_b():
    """3-D: triangular prisms from base/height and from vertices, a trapezoidal prism, a TERS
    tip, a regular tetrahedron and one from real-space vertices; Ex plane source, flux box,
    two BIN planes."""
    cfg = configs.config2(n=44, pml=6, steps=200, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    lor = configs.drude_lorentz_pols(5.0, [(0.6, 0.3, 2.4)])
    verts = [{"vert": [0.01, 0.16]}, {"vert": [0.15, -0.1]}, {"vert": [-0.13, -0.07]}]
    tet = [{"vert": [0.31, 0.17, -0.12]}, {"vert": [0.57, 0.23, -0.06]}, {"vert": [0.41, 0.46, 0.01]},
           {"vert": [0.43, 0.29, 0.21]}]
    cfg["ObjectList"] = [
        _shape("triangle_prism", [-0.4, -0.3, 0.0], 2.0, base=0.3, height=0.26, length=0.3, unit_vectors=_rot(20.0, 30.0)),
        _shape("triangle_prism", [0.0, -0.3, 0.02], 2.6, vertLocs=verts, length=0.25),
        _shape("trapezoid_prism", [0.4, -0.3, 0.0], 1.7, pols=lor, base1=0.3, base2=0.14, height=0.21, length=0.26,
               orPhi=15.0),
        _shape("ters_tip", [-0.4, 0.3, 0.0], 3.2, rad_curve=0.1, base=0.3, length=0.3),
        _shape("tetrahedron", [0.0, 0.3, 0.0], 2.4, sideLen=0.34, unit_vectors=_rot(15.0, 35.0)),
        _shape("tetrahedron", [0.0, 0.0, 0.0], 1.9, vertLocs=tet),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Ey", (0.0, 1.5, 1.5))])


def _shapes_2d():
    """2-D TMz: partial torus, paraboloid, hemisphere, rounded block and triangular prism (in
    2-D the third unit vector is zero, so the reference's object-frame z is NaN and every test
    on it passes: the torus fills its azimuth range and the paraboloid a half-plane, so they
    come first and the others overwrite them); point source, text detectors, flux line, one
    BIN plane."""
    cfg = configs.config1(n=80, pml=10, steps=300, radius_cells=10, src_gap_cells=12, ndtc=3, nfreq=8)
    cfg["ObjectList"] = [
        _shape("torus", [-0.6, -0.6, 0.0], 1.8, rad_Ring=0.25, rad_CrossSec=0.1, phiMin=0.0, phiMax=250.0),
        _shape("paraboloid", [0.0, 0.0, 0.0], 2.2, a=0.5, b=0.4, length=0.5, orPhi=90.0),
        _shape("hemisphere", [0.5, 0.6, 0.0], 2.0, radius=0.3, orPhi=45.0),
        _shape("block", [-0.6, 0.7, 0.0], 2.5, size=[0.6, 0.4, 0.0], rad_curve=0.1, orPhi=20.0),
        _shape("triangle_prism", [0.7, -0.6, 0.0], 3.0, base=0.5, height=0.45, length=0.0, orPhi=-30.0),
    ]
    return _bin_planes(cfg, [("Ez", (3.0, 3.0, 0.0))])


def _named(shape, loc, material, **kw):
    return configs._obj(shape, loc, material=material, **kw)


def _named_3d():
    """3-D: named materials (Rakic Au and W, JM Ag, TiO2, Si, the CdSe quantum-dot
    resonance); Ex plane source, flux box, two BIN planes."""
    cfg = configs.config2(n=44, pml=6, steps=220, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    cfg["ObjectList"] = [
        _named("block", [-0.35, -0.3, 0.0], "TiO2", size=[0.3, 0.25, 0.3]),
        _named("sphere", [0.0, 0.0, 0.0], "Au", radius=0.18),
        _named("ellipsoid", [0.38, -0.3, 0.05], "JM_Ag", size=[0.3, 0.2, 0.24]),
        _named("cylinder", [-0.35, 0.35, 0.0], "CdSeQD", radius=0.12, length=0.3),
        _named("sphere", [0.38, 0.35, 0.0], "Si", radius=0.13),
        _named("hemisphere", [0.0, -0.45, 0.0], "w", radius=0.12),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Ey", (0.0, 1.5, 1.5))])


def _named_2d():
    """2-D TMz: Rakic Ag and Al, JM Au and Sn, the PbS quantum-dot resonance, SiO2; point
    source, text detectors, flux line, one BIN plane."""
    cfg = configs.config1(n=80, pml=10, steps=300, radius_cells=10, src_gap_cells=12, ndtc=3, nfreq=8)
    cfg["ObjectList"] = [
        _named("sphere", [0.0, 0.0, 0.0], "AG", radius=0.35),
        _named("block", [0.8, 0.6, 0.0], "JM_Au", size=[0.4, 0.3, 0.0]),
        _named("block", [-0.8, 0.6, 0.0], "al", size=[0.3, 0.5, 0.0]),
        _named("sphere", [0.7, -0.7, 0.0], "PbSQD", radius=0.2),
        _named("sphere", [-0.7, -0.7, 0.0], "JM_sn", radius=0.2),
        _named("block", [0.0, 1.0, 0.0], "SiO2", size=[0.8, 0.2, 0.0]),
    ]
    return _bin_planes(cfg, [("Ez", (3.0, 3.0, 0.0))])


def _src(pol, loc, size, pulse, phi=None, **kw):
    s = {"pol": pol, "loc": loc, "size": size, "PulseList": [pulse]}
    if phi is not None:
        s["phi"] = phi
    s.update(kw)
    return s


def _src_oblique_2d():
    """2-D TMz: an Ez line source at phi = 30 degrees (an oblique source: every cell adds the
    pulse delayed by its distance along the direction of travel) onto the dielectric disk."""
    cfg = configs.config1(n=72, pml=8, steps=260, radius_cells=7, src_gap_cells=8, ndtc=3, nfreq=8)
    pulse = cfg["SourceList"][0]["PulseList"][0]
    cfg["SourceList"] = [_src("Ez", [-0.8, -0.2, 0.0], [1.0, 0.0, 0.0], pulse, phi=30)]
    return cfg


def _src_oblique_te():
    """2-D TE (Ex, Ey, Hz): an oblique Ey line source at phi = 60 degrees (it acts on Ex and
    Ey) and an oblique Hz line source at phi = -45 degrees, onto a Drude-Lorentz disk."""
    cfg = configs.config1(n=72, pml=8, steps=260, radius_cells=7, src_gap_cells=8, ndtc=3, nfreq=8)
    cfg["CompCell"]["pol"] = "Hz"
    pulse = cfg["SourceList"][0]["PulseList"][0]
    cfg["SourceList"] = [_src("Ey", [-0.7, -0.5, 0.0], [0.8, 0.0, 0.0], pulse, phi=60),
                         _src("Hz", [0.6, 0.7, 0.0], [0.6, 0.0, 0.0], pulse, phi=-45)]
    cfg["ObjectList"][0]["pols"] = configs.drude_lorentz_pols(4.0, [(1.0, 0.2, 0.0), (0.6, 0.3, 2.4)])
    for d in cfg["DetectorList"]:
        d["type"] = "Hz"
    cfg["DetectorList"].append({"loc": [0.3, -0.4, 0.0], "size": [0.0, 0.0, 0.0], "type": "Ex",
                                "fname": "out/te_ex", "dtc_class": "txt", "SI": False, "Time_Interval": cfg["CompCell"]["dt"]})
    return cfg


def _src_3d(srcs):
    cfg = configs.config2(n=30, pml=5, steps=150, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    width = 0.3e-15 / configs.T_UNIT
    pulse = configs._gauss(configs.A / 550e-9, 1.0 / width, 4.0, 2 * width)
    cfg["SourceList"] = [_src(pol, loc, size, pulse, **kw) for pol, loc, size, kw in srcs]
    cfg["ObjectList"] = [configs._obj("sphere", [0.05, 0.0, 0.1], radius=0.2, material="custom", eps=2.5,
                                      pols=configs.drude_lorentz_pols(3.0, [(0.8, 0.3, 2.2)]))]
    cfg["DetectorList"].append({"loc": [0.2, -0.15, 0.3], "size": [0.0, 0.0, 0.0], "type": "Ez",
                                "fname": "out/c2_ez", "dtc_class": "txt", "SI": False, "Time_Interval": cfg["CompCell"]["dt"]})
    return cfg


def _src_oblique_3d():
    """3-D: oblique Ez and Hx sheets (phi = 45 and 120 degrees). The reference reads no polar
    angle for soft sources, so in 3-D the plane of an oblique source is normal to z."""
    return _src_3d([("Ez", [0.0, 0.0, -0.4], [0.5, 0.5, 0.0], {"phi": 45}),
                    ("Hx", [0.1, -0.1, -0.3], [0.4, 0.4, 0.0], {"phi": 120})])


def _src_circ_3d():
    """3-D: a left circularly polarised xy sheet (Ex and Ey) and a right circularly polarised
    yz sheet (Ey and Ez) with polarisation angles and an axis ratio."""
    return _src_3d([("L", [0.0, 0.0, -0.4], [0.6, 0.6, 0.0], {"psi": 30.0}),
                    ("R", [-0.45, 0.0, 0.0], [0.0, 0.5, 0.4], {"psi": 10.0, "ellpiticalKRat": 0.5})])


def _relpole(kind, strength=1.5, **angles):
    """A Lorentz pole whose dipole is set relative to the local surface of its object."""
    pole = {"gamma": 0.01, "omega": 5.0 * configs.A / 550e-9, "sigma_p": strength, "dipOrE": kind}
    pole.update(angles)
    return pole


def _dip_surface_a():
    """3-D: Lorentz poles with dipoles relative to the surface: normal on a sphere, at 30
    degrees from the normal (azimuth 60) on a rotated ellipsoid, tangent on a rotated block,
    longitudinal-tangent (which the reference leaves at zero) next to a normal pole on a
    cylinder, tangent on a hemisphere; Ex plane source, flux box, two BIN planes."""
    cfg = configs.config2(n=44, pml=6, steps=200, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    cfg["ObjectList"] = [
        _shape("sphere", [-0.4, 0.3, 0.0], 1.6, pols=[_relpole("normal")], radius=0.15),
        _shape("ellipsoid", [0.0, 0.3, 0.05], 1.8, pols=[_relpole("rel_norm", polAngRelNormE=30.0, azAngRelNormE=60.0)],
               size=[0.34, 0.22, 0.28], unit_vectors=_rot(25.0, 40.0)),
        _shape("block", [0.4, 0.3, 0.0], 2.0, pols=[_relpole("tangent", 2.0)], size=[0.26, 0.22, 0.3],
               unit_vectors=_rot(15.0, 20.0)),
        _shape("cylinder", [-0.3, -0.3, 0.0], 1.5, pols=[_relpole("long_tangent"), _relpole("normal", 1.0)],
               radius=0.12, length=0.3, orTheta=70.0, orPhi=25.0),
        _shape("hemisphere", [0.3, -0.3, 0.0], 1.7, pols=[_relpole("tangent")], radius=0.16, orPhi=30.0),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Ey", (0.0, 1.5, 1.5))])


def _dip_surface_b():
    """3-D: surface-relative dipoles on a cone, a partial torus, a paraboloid, a rounded block
    (corner and face normals), a hemiellipsoid, a regular tetrahedron and one from vertices;
    Ex plane source, flux box, two BIN planes."""
    cfg = configs.config2(n=44, pml=6, steps=200, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    tet = [{"vert": [0.31, 0.17, -0.12]}, {"vert": [0.57, 0.23, -0.06]}, {"vert": [0.41, 0.46, 0.01]},
           {"vert": [0.43, 0.29, 0.21]}]
    cfg["ObjectList"] = [
        _shape("cone", [-0.4, 0.35, 0.0], 1.4, pols=[_relpole("normal")], radSmall=0.05, radLarge=0.15, height=0.3),
        _shape("torus", [0.0, 0.3, -0.05], 1.6, pols=[_relpole("rel_norm", polAngRelNormE=60.0, azAngRelNormE=20.0)],
               rad_Ring=0.13, rad_CrossSec=0.06, phiMin=20.0, phiMax=290.0, unit_vectors=_rot(30.0, 0.0)),
        _shape("paraboloid", [0.4, 0.3, 0.0], 1.8, pols=[_relpole("normal")], a=0.28, b=0.2, length=0.3,
               orTheta=60.0, orPhi=20.0),
        _shape("block", [-0.4, -0.3, 0.0], 2.0, pols=[_relpole("normal")], size=[0.3, 0.26, 0.22], rad_curve=0.06,
               unit_vectors=_rot(10.0, 15.0)),
        _shape("hemiellipsoid", [0.0, -0.3, 0.05], 1.9, pols=[_relpole("tangent")], size=[0.3, 0.22, 0.26],
               unit_vectors=_rot(25.0, 40.0)),
        # the regular tetrahedron's height cut-off is taken at twice its location (the
        # reference adds the location to a vertex that already holds it), so it sits at the
        # origin; its material index is tested against its two-entry size, which no point
        # passes, so its pole has no cells (its permittivity does)
        _shape("tetrahedron", [0.0, 0.0, 0.0], 2.2, pols=[_relpole("tangent")], sideLen=0.34,
               unit_vectors=_rot(15.0, 35.0)),
        _shape("tetrahedron", [0.0, 0.0, 0.0], 1.7, pols=[_relpole("normal")], vertLocs=tet),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Ey", (0.0, 1.5, 1.5))])


def _level(e_cen_ev, dist, nstates, width_ev, **factors):
    lv = configs.emitter_level(e_cen_ev, dist, nstates, width_ev)
    lv.update({k: [v] for k, v in factors.items()})
    return lv


def _qe_dists_3d():
    """qe_3d's three-level ladder with a skew-normal (skew 2) and an exponential-power
    (shape 1.5) broadened upper level, three sampled energies each."""
    cfg = _qe_3d()
    lv = [configs.emitter_level(0.0), _level(2.0, "skew_normal", 3, 0.02, skew_factor=2.0),
          _level(4.2, "exp_pow", 3, 0.02, shape_factor=1.5)]
    cfg["ObjectList"][0]["Energy_Levels"] = lv
    return cfg


def _qe_dists_2d():
    """qe_tm's two-level block with a generalised skew-normal (shape 0.3) broadened upper
    level sampled at four energies."""
    cfg = _qe_tm()
    lv = [configs.emitter_level(0.0), _level(2.0, "gen_skew_normal", 4, 0.03, shape_factor=0.3)]
    o = cfg["ObjectList"][0]
    o["Energy_Levels"] = lv
    n = 2
    o["couplings"] = [1e5] * (n * n)
    return cfg


def _layer_scene(layers, m=(0, 0, 1), theta=0.0, phi=90.0, psi=0.0, n=36, steps=200, sphere=None, det="Ex"):
    """3-D TFSF box (4 cells inside the CPML) with material layers (block objects that
    span the cell across the propagation axis) crossing its side surfaces; the flux box
    and a point detector of component ``det`` sit inside the box. ``layers``: (lo, hi,
    eps, pols) along the propagation axis, in a units; ``sphere``: (centre, radius, eps),
    a scatterer inside the flux box, so that every face of the flux box carries scattered
    power and not only rounding noise."""
    cfg = configs.config2(n=n, pml=6, steps=steps, nell=0, nfreq=5, metal_radius_cells=0, tfsf=True)
    cfg["DetectorList"][0]["type"] = det
    axis = [i for i in range(3) if m[i] != 0][0]
    size = cfg["CompCell"]["size"][0]
    objs = []
    if sphere is not None:
        objs.append(_shape("sphere", sphere[0], sphere[2], radius=sphere[1]))
    for lo, hi, eps, pols in layers:
        loc = [0.0, 0.0, 0.0]
        sz = [2 * size, 2 * size, 2 * size]
        loc[axis] = (lo + hi) / 2
        sz[axis] = hi - lo
        objs.append(_shape("block", loc, eps, pols, size=sz))
    cfg["ObjectList"] = objs
    t = cfg["TFSF"][0]
    width = 0.2e-15 / configs.T_UNIT
    t["PulseList"] = [configs._gauss(configs.A / 550e-9, 1.0 / width, 4.0, 2 * width)]
    t["pmlThick"] = 8
    t["m"] = list(m)
    t["theta"], t["phi"], t["psi"] = theta, phi, psi
    return cfg


def _tfsf_layer_3d():
    """Normal incidence along +z onto a dielectric substrate (eps 2.25) whose face lies
    inside the TFSF box: the incident lines are layered, the surface terms inside the
    substrate are divided by its eps."""
    return _layer_scene([(0.1, 2.0, 2.25, [])], sphere=([0.03, 0.0, -0.11], 0.15, 3.0))


def _tfsf_film_3d():
    """Normal incidence along +z onto a Drude-Lorentz film (eps_inf 2) on a dielectric
    substrate, both crossing the box sides: the lines carry the film's poles and the
    corrections inside the film go to D."""
    film = configs.drude_lorentz_pols(9.0, [(1.0, 0.07, 0.0), (1.0, 0.4, 2.6)])
    return _layer_scene([(0.0, 0.2, 2.0, film), (0.2, 2.0, 1.8, [])], sphere=([0.03, 0.0, -0.15], 0.13, 3.0))


def _tfsf_layer_x():
    """Normal incidence along +x (Ey) onto a Lorentz layer and a dielectric substrate."""
    lor = configs.drude_lorentz_pols(3.0, [(0.6, 0.3, 3.2)])
    return _layer_scene([(-0.05, 0.1, 1.5, lor), (0.25, 2.0, 2.5, [])], m=(1, 0, 0), theta=90.0, phi=0.0,
                        sphere=([-0.19, 0.03, 0.0], 0.12, 3.0), det="Ey")


def _mu_3d():
    """3-D: constant-mu objects away from the CPML: a dielectric sphere with mu 1.5, a
    mu-only block (eps 1, mu 2.5) and a Lorentz cylinder with mu 1.3; Ex plane source, flux
    box, two BIN planes (an H plane among them)."""
    cfg = configs.config2(n=44, pml=6, steps=200, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    lor = configs.drude_lorentz_pols(5.0, [(0.6, 0.3, 2.4)])
    cfg["ObjectList"] = [
        _shape("sphere", [-0.3, -0.25, 0.0], 2.0, radius=0.15, mu=1.5),
        _shape("block", [0.25, -0.2, 0.05], 1.0, size=[0.3, 0.26, 0.22], mu=2.5),
        _shape("cylinder", [0.0, 0.3, 0.0], 1.6, pols=lor, radius=0.12, length=0.3, mu=1.3),
    ]
    return _bin_planes(cfg, [("Ex", (1.5, 1.5, 0.0)), ("Hy", (0.0, 1.5, 1.5))])


def _mu_2d():
    """2-D TMz: a disk with mu 2 and eps 1.5 and a mu-only disk; point source, text
    detectors, flux line, one BIN plane of Hx."""
    cfg = configs.config1(n=80, pml=10, steps=300, radius_cells=10, src_gap_cells=12, ndtc=3, nfreq=8)
    cfg["ObjectList"] = [
        _shape("sphere", [-0.3, 0.2, 0.0], 1.5, radius=0.25, mu=2.0),
        _shape("sphere", [0.35, -0.3, 0.0], 1.0, radius=0.2, mu=1.8),
    ]
    return _bin_planes(cfg, [("Hx", (3.0, 3.0, 0.0))])


CASES = {
    "c1_small": lambda: configs.config1(n=80, pml=10, steps=300, radius_cells=10, src_gap_cells=12, ndtc=4, nfreq=12),
    "c2_small": lambda: configs.config2(n=34, pml=6, steps=70, nell=3, nfreq=6, metal_radius_cells=20, aniso=False,
                                          tfsf=False),
    "c2_aniso": _c2_aniso,
    "te_dispersive": _te_dispersive,
    "tm_lorentz": _tm_lorentz,
    "qe_tm": _qe_tm,
    "qe_te": _qe_te,
    "qe_3d": _qe_3d,
    "tfsf_disp": _tfsf_disp,
    "tfsf_oblique": _tfsf_oblique,
    "tfsf_2d_te": _tfsf_2d_te,
    "freq_3d": _freq_3d,
    "freq_2d": _freq_2d,
    "c5_small": _c5_small,
    "shapes_a": _shapes_a,
    "shapes_b": _shapes_b,
    "shapes_2d": _shapes_2d,
    "named_3d": _named_3d,
    "named_2d": _named_2d,
    "flux_save": lambda: _flux_scene(save=True),
    "flux_load": lambda: _flux_scene(load="incident_fields.dat"),
    "src_oblique_2d": _src_oblique_2d,
    "src_oblique_te": _src_oblique_te,
    "src_oblique_3d": _src_oblique_3d,
    "src_circ_3d": _src_circ_3d,
    "dip_surface_a": _dip_surface_a,
    "dip_surface_b": _dip_surface_b,
    "qe_dists_3d": _qe_dists_3d,
    "qe_dists_2d": _qe_dists_2d,
    "tfsf_layer_3d": _tfsf_layer_3d,
    "tfsf_film_3d": _tfsf_film_3d,
    "tfsf_layer_x": _tfsf_layer_x,
    "mu_3d": _mu_3d,
    "mu_2d": _mu_2d,
}


def _qe_two_objects():
    """Two emitter objects (the qe_tm block and a disk of two-level emitters). The reference
    pools every emitter object's energy levels into one list (qeELevs_) and builds each
    object's Hamiltonians from it, so the first object's Hamiltonian diagonal no longer
    matches its ensemble energies and parallelQE's constructor throws."""
    cfg = _qe_tm()
    lv = [configs.emitter_level(0.0), configs.emitter_level(2.1)]
    cfg["ObjectList"].append(configs.emitter_obj("sphere", [0.4, 0.3, 0.0], [(0, 0), (1, 0)], lv, [1e5] * 4,
                                                 [(1, 0, 1e12, 2e13)], 1e21, eps=1.2, dtc_levs=[3],
                                                 output_pol="out/qe2_pol.dat", radius=0.15))
    return cfg


def _ordip_2d(pol):
    """A 2-D disk with one unidirectional (oriented-dipole) pole; the reference stops on a
    grid index assertion while it builds the oriented-dipole lists in 2-D."""
    def make():
        cfg = configs.config1(n=60, pml=8, steps=200, radius_cells=8, src_gap_cells=6, ndtc=2, nfreq=4)
        cfg["CompCell"]["pol"] = pol
        if pol == "Hz":
            cfg["SourceList"][0]["pol"] = "Ey"
            for d in cfg["DetectorList"]:
                d["type"] = "Ey"
        cfg["ObjectList"][0]["pols"] = [{"gamma": 0.01, "omega": 5.0 * configs.A / 550e-9, "sigma_p": 1.5,
                                         "dipOrE": "unidirectional", "dirDipE": [0.6, 0.8, 0.0]}]
        return cfg
    return make


def _flux_scene(objects=True, save=False, load=None):
    """3-D: a dielectric sphere (eps 2.5) in a 30^3 cell, an Ex plane source below it, a flux
    box around it; optionally saving the flux fields, or loading incident fields."""
    cfg = configs.config2(n=30, pml=5, steps=160, nell=0, nfreq=5, metal_radius_cells=0, tfsf=False)
    width = 0.3e-15 / configs.T_UNIT
    cfg["SourceList"][0]["PulseList"] = [configs._gauss(configs.A / 550e-9, 1.0 / width, 4.0, 2 * width)]
    cfg["ObjectList"] = [configs._obj("sphere", [0.0, 0.0, 0.0], radius=0.15, material="custom", eps=2.5, pols=[])] if objects else []
    fl = cfg["FluxList"][0]
    if save:
        fl["save"] = True
    if load:
        fl["load"] = True
        fl["incd_fileds"] = load
    return cfg


# Files a case needs beside its input, made by a reference run of another input: the
# case's inputs/ directory holds them, and runs of the case start with them in their
# working (output) directory.
INPUT_FILES = {
    "flux_load": ("incident_fields.dat", lambda: _flux_scene(objects=False, save=True), "out/c2_flux_fields.dat"),
}


# Inputs the reference build does not finish: <case>/ref_error.txt keeps the last line it
# printed, and the engine must reject the input instead of running it.
def _tfsf_layer_oblique():
    """A substrate crossing the box under oblique incidence: the reference allows material
    changes across the surfaces only for normal incidence (genEpMu throws)."""
    return _layer_scene([(0.1, 2.0, 2.25, [])], m=(1, 0, 1), theta=45.0, phi=0.0)


def _tfsf_sphere_cross():
    """A sphere crossing the side surfaces: its slices across the propagation are not
    uniform, which genEpMu refuses."""
    cfg = _layer_scene([])
    cfg["ObjectList"] = [_shape("sphere", [0.0, 0.3, 0.0], 2.0, radius=0.2)]
    return cfg


def _tfsf_layer_2d():
    """2-D TE along +y onto a substrate: the normal plane fills the whole line first, so
    the layered side plane disagrees with it and genEpMu throws."""
    cfg = _tfsf_2d_te()
    cfg["TFSF"][0]["m"] = [0, 1, 0]
    cfg["TFSF"][0]["theta"], cfg["TFSF"][0]["phi"] = 90.0, 90.0
    cfg["ObjectList"] = [_shape("block", [0.0, 1.0, 0.0], 2.0, size=[6.0, 2.0, 0.0])]
    return cfg


FAILING = {
    "tfsf_layer_oblique": _tfsf_layer_oblique,
    "tfsf_sphere_cross": _tfsf_sphere_cross,
    "tfsf_layer_2d": _tfsf_layer_2d,
    "qe_two_objects": _qe_two_objects,
    "ordip_2d_tm": _ordip_2d("Ez"),
    "ordip_2d_te": _ordip_2d("Hz"),
}


def main(names=None):
    ref = os.path.join(ROOT, "oracle", "_ref", "chiml_ref")
    if not os.path.exists(ref):
        raise SystemExit("build the reference first: make -f oracle/Makefile.ref")
    for name, make in CASES.items():
        if names and name not in names:
            continue
        case = os.path.join(HERE, name)
        shutil.rmtree(case, ignore_errors=True)
        os.makedirs(case)
        configs.write_json(make(), os.path.join(case, "in.json"))
        staged = []
        if name in INPUT_FILES:
            fname, make_src, produced = INPUT_FILES[name]
            with tempfile.TemporaryDirectory() as tmp:
                configs.write_json(make_src(), os.path.join(tmp, "in.json"))
                r = subprocess.run([ref, "in.json"], cwd=tmp, capture_output=True, text=True)
                if r.returncode != 0:
                    raise SystemExit("%s (input file) failed:\n%s%s" % (name, r.stdout, r.stderr))
                os.makedirs(os.path.join(case, "inputs"))
                shutil.copy(os.path.join(tmp, produced), os.path.join(case, "inputs", fname))
            staged = [fname]
        with tempfile.TemporaryDirectory() as tmp:
            shutil.copy(os.path.join(case, "in.json"), os.path.join(tmp, "in.json"))
            for fname in staged:
                shutil.copy(os.path.join(case, "inputs", fname), os.path.join(tmp, fname))
            r = subprocess.run([ref, "in.json"], cwd=tmp, capture_output=True, text=True)
            if r.returncode != 0:
                raise SystemExit("%s failed:\n%s%s" % (name, r.stdout, r.stderr))
            for d, _, files in os.walk(tmp):
                for f in files:
                    src = os.path.join(d, f)
                    rel = os.path.relpath(src, tmp)
                    if rel == "in.json" or f == "levelDist.dat" or rel in staged:
                        continue
                    dst = os.path.join(case, "ref", rel)
                    os.makedirs(os.path.dirname(dst), exist_ok=True)
                    shutil.copy(src, dst)
        print(name, "ok")
    for name, make in FAILING.items():
        if names and name not in names:
            continue
        case = os.path.join(HERE, name)
        shutil.rmtree(case, ignore_errors=True)
        os.makedirs(case)
        configs.write_json(make(), os.path.join(case, "in.json"))
        with tempfile.TemporaryDirectory() as tmp:
            shutil.copy(os.path.join(case, "in.json"), os.path.join(tmp, "in.json"))
            r = subprocess.run([ref, "in.json"], cwd=tmp, capture_output=True, text=True)
            if r.returncode == 0:
                raise SystemExit("%s: the reference finished; it is expected to fail" % name)
            last = (r.stderr.strip().splitlines() or ["exit status %d" % r.returncode])[-1]
            # the reference's own source path in an assertion message is not part of the record
            last = last.replace(os.path.join(os.environ.get("CHIML_REF_SRC", ""), ""), "")
            with open(os.path.join(case, "ref_error.txt"), "w") as f:
                f.write("exit status %d\n%s\n" % (r.returncode, last))
        print(name, "fails in the reference, as expected")


if __name__ == "__main__":
    main(sys.argv[1:])

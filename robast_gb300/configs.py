"""Scene and ray-batch builders for the benchmark configurations.

Each builder returns (manager, batch) where batch holds host ray arrays
(x, y, z, dx, dy, dz, lam, group) produced with the ARayShooter laws; group
is the field-angle / variant index of each ray for the spot reductions.
All inputs are synthetic and seeded.

  paraboloid          single paraboloid mirror (tutorials/SimpleParabolicTelescope.C)
  davies_cotton       380 hexagonal spherical facets (tutorials/DaviesCotton.C)
  schwarzschild_couder two AGeoAsphericDisk mirrors (tutorials/SchwarzschildCouder.C)
  light_guide         7x7 hexagonal AGeoWinstonConePoly behind an ALens window
  schmidt_cassegrain  corrector + spherical primary/secondary with a 20-layer stack
"""
from __future__ import annotations

import math
from typing import Dict, Tuple

import numpy as np

from .geometry import (AGeoAsphericDisk, AGeoWinstonConePoly, TGeoBBox, TGeoCombiTrans, TGeoCompositeShape,
                       TGeoParaboloid, TGeoPgon, TGeoRotation, TGeoSphere, TGeoTranslation, TGeoTube)
from .manager import AOpticsManager, ARayArray, ARayShooter
from .optics import (ABorderSurfaceCondition, AFocalSurface, ALens, AMirror, AMultilayer, AObscuration,
                     AOpticalComponent, ARefractiveIndex, ASellmeierFormula, TGraph)

cm, m, mm, um, nm = 1.0, 100.0, 0.1, 1e-4, 1e-7
deg = math.pi / 180.0


def _concat(batches):
    out = {}
    for k in batches[0]:
        out[k] = np.concatenate([b[k] for b in batches])
    return out


def _batch(arr: ARayArray, group: int) -> Dict[str, np.ndarray]:
    n = len(arr)
    return {"x": arr.x, "y": arr.y, "z": arr.z, "dx": arr.dx, "dy": arr.dy, "dz": arr.dz, "lam": arr.lam,
            "group": np.full(n, group, dtype=np.int32)}


def to_array(batch) -> ARayArray:
    return ARayArray.from_arrays(batch["x"], batch["y"], batch["z"], batch["dx"], batch["dy"], batch["dz"],
                                 batch["lam"])


def _split(n, k):
    base = [n // k] * k
    for i in range(n % k):
        base[i] += 1
    return base


# ---------------------------------------------------------------------------
# 1. paraboloid (tutorials/SimpleParabolicTelescope.C:22-83)
# ---------------------------------------------------------------------------
def paraboloid(n_rays: int = 1_000_000, angles=(0.0, 0.5, 1.0, 2.0), seed: int = 1):
    F = 8 * m
    R = 1 * m
    sag = R * R / 4.0 / F
    Rf = 30 * cm
    man = AOpticsManager("manager", "paraboloid")
    world = AOpticalComponent("world", TGeoBBox("worldbox", 20 * m, 20 * m, 20 * m))
    man.SetTopVolume(world)
    para = TGeoParaboloid("mirror_para", 0, R, sag / 2.0)
    tr1 = TGeoTranslation("mirror_tr1", 0, 0, sag / 2.0).RegisterYourself()
    tr2 = TGeoTranslation("mirror_tr2", 0, 0, sag / 2.0 - 1 * um).RegisterYourself()
    comp = TGeoCompositeShape("mirror_comp", "mirror_para:mirror_tr2 - mirror_para:mirror_tr1")
    mirror = AMirror("mirror", comp)
    mirror.SetReflectance(1.0)
    world.AddNode(mirror, 1)
    focal = AFocalSurface("focal", TGeoTube("focal_tube", 0, Rf, 10 * um))
    world.AddNode(focal, 1, TGeoTranslation("focal_tr", 0, 0, F + 10 * um))
    obs1 = AObscuration("obs1", TGeoTube("obs_tube1", 0, Rf + 10 * um, 10 * um))
    world.AddNode(obs1, 1, TGeoTranslation("obs_tr1", 0, 0, F + 30 * um))
    obs2 = AObscuration("obs2", TGeoTube("obs_tube2", Rf, Rf + 10 * um, 10 * um))
    world.AddNode(obs2, 1, TGeoTranslation("obs_tr2", 0, 0, F + 10 * um))
    man.CloseGeometry()
    batches = []
    for g, (a, n) in enumerate(zip(angles, _split(n_rays, len(angles)))):
        r = a * deg
        tr = TGeoTranslation(-2 * F * math.sin(r), 0, 2 * F * math.cos(r))
        v = (math.sin(r), 0.0, -math.cos(r))
        arr = ARayShooter.RandomCircle(400 * nm, 110 * cm, n, None, tr, v, seed=seed * 1000 + g)
        batches.append(_batch(arr, g))
    return man, _concat(batches)


# ---------------------------------------------------------------------------
# 3. Schwarzschild-Couder (tutorials/SchwarzschildCouder.C:19-81, OS2 design)
# ---------------------------------------------------------------------------
SC_FP = 16.915 * m
SC_FS = -3.553 * m
SC_FF = -1.481 * m
SC_ZS = 9.980 * m
SC_ZF = 7.631 * m
SC_PRIMARY_K = [SC_FP ** -1 * 0.25, SC_FP ** -3 * -0.189377, SC_FP ** -5 * -0.604706, SC_FP ** -7 * -4.21374,
                SC_FP ** -9 * 21.8275, SC_FP ** -11 * -425.160, 0.0, 0.0]
SC_SECONDARY_K = [SC_FS ** -1 * 0.25, SC_FS ** -3 * 0.013625, SC_FS ** -5 * -0.010453, SC_FS ** -7 * 0.014241,
                  SC_FS ** -9 * -0.012213, SC_FS ** -11 * 0.005184, 0.0, 0.0]


def schwarzschild_couder(n_rays: int = 10_000_000, angles=(0.0, 1.0, 2.0, 3.0, 4.0), seed: int = 3,
                         perturb: float = 1e-3, primary_k=None, secondary_k=None,
                         secondary_shift=(0.0, 0.0, 0.0), secondary_tilt=(0.0, 0.0)):
    """Primary 9.7 m / 4.4 m (outer / inner diameter), secondary 5.4 m, both
    1-um thick AGeoAsphericDisks with the same 8-term polynomial on both
    faces; OS2 coefficients perturbed by N(0, perturb) relative (seeded)."""
    rng = np.random.default_rng(seed)
    kp = np.array(SC_PRIMARY_K if primary_k is None else primary_k, dtype=float)
    ks = np.array(SC_SECONDARY_K if secondary_k is None else secondary_k, dtype=float)
    if primary_k is None and perturb:
        kp = kp * (1 + perturb * rng.standard_normal(8))
    if secondary_k is None and perturb:
        ks = ks * (1 + perturb * rng.standard_normal(8))
    man = AOpticsManager("manager", "SC")
    world = AOpticalComponent("world", TGeoBBox("worldbox", 30 * m, 30 * m, 30 * m))
    man.SetTopVolume(world)
    top = AOpticalComponent("top", TGeoBBox("topbox", 30 * m, 30 * m, 30 * m))
    primaryV = AGeoAsphericDisk("primaryV", -1 * um, 0, 0 * m, 0, 9.7 * m / 2.0, 4.4 * m / 2.0)
    primaryV.SetPolynomials(8, kp, 8, kp)
    primary = AMirror("primaryMirror", primaryV)
    top.AddNode(primary, 1)
    secondaryV = AGeoAsphericDisk("secondaryV", SC_ZS, 0, SC_ZS + 1 * um, 0, 5.4 * m / 2.0, 0 * m)
    secondaryV.SetPolynomials(8, ks, 8, ks)
    secondary = AMirror("secondaryMirror", secondaryV)
    if any(secondary_shift) or any(secondary_tilt):
        rot = TGeoRotation("", 0, 0, 0)
        rot.RotateX(secondary_tilt[0] / deg)
        rot.RotateY(secondary_tilt[1] / deg)
        if len(secondary_tilt) > 2:
            rot.RotateZ(secondary_tilt[2] / deg)
        # rotate about the mirror vertex (z = SC_ZS)
        c = np.array([0.0, 0.0, SC_ZS])
        t = c - rot.R @ c + np.asarray(secondary_shift, dtype=float)
        top.AddNode(secondary, 1, TGeoCombiTrans(t[0], t[1], t[2], rot))
    else:
        top.AddNode(secondary, 1)
    ky = [SC_FF ** -1 * 0.25]
    focalV = AGeoAsphericDisk("focalV", SC_ZF - 1 * mm, 0, SC_ZF, 0, 1 * m, 0.0)
    focalV.SetPolynomials(1, ky, 1, ky)
    focal = AFocalSurface("focalPlane", focalV)
    top.AddNodeOverlap(focal, 1)
    f1 = focalV.CalcF1(1 * m)
    obsV = AGeoAsphericDisk("focalObsV", f1 - 1 * cm, 0, f1, 0, 1 * m * 1.043, 0.0)
    obs = AObscuration("focalObs", obsV)
    top.AddNodeOverlap(obs, 1)
    world.AddNode(top, 1)
    man.CloseGeometry()
    batches = []
    for g, (a, n) in enumerate(zip(angles, _split(n_rays, len(angles)))):
        r = a * deg
        tr = TGeoTranslation(-1.2 * SC_ZS * math.sin(r), 0, 1.2 * SC_ZS * math.cos(r))
        rot = TGeoRotation("", -90.0, a, 90.0)  # disk perpendicular to the beam
        arr = ARayShooter.RandomCircle(400 * nm, 5 * m, n, rot, tr, (0.0, 0.0, -1.0), seed=seed * 1000 + g)
        batches.append(_batch(arr, g))
    return man, _concat(batches)


def plate_scale_sc():
    """cm on the focal surface per degree of field (10 cm per degree for OS2
    as used by tutorials/SchwarzschildCouder.C:148)."""
    return 10 * cm


# ---------------------------------------------------------------------------
# 2. Davies-Cotton (tutorials/DaviesCotton.C:30-160)
# ---------------------------------------------------------------------------
def _hex_lattice(pitch, n):
    """The n hexagonal-lattice sites nearest the origin (flat-to-flat pitch)."""
    k = int(math.ceil(math.sqrt(n))) + 4
    pts = []
    for i in range(-k, k + 1):
        for j in range(-k, k + 1):
            x = pitch * (i + 0.5 * j)
            y = pitch * (math.sqrt(3) / 2.0) * j
            pts.append((x * x + y * y, x, y))
    pts.sort()
    return [(x, y) for _, x, y in pts[:n]]


def davies_cotton(n_rays: int = 10_000_000, n_angles: int = 11, max_angle: float = 2.5, seed: int = 2,
                  n_facets: int = 380, tilt_sigma: float = 0.5e-3, roughness: float = 1e-3):
    F = 15 * m
    Rc = 2 * F
    D = 60 * cm  # facet flat-to-flat
    T = 0.1 * mm
    rng = np.random.default_rng(seed)
    man = AOpticsManager("manager", "Davies-Cotton System")
    man.DisableFresnelReflection(True)
    world = AOpticalComponent("world", TGeoBBox("boxWorld", 20 * m, 20 * m, 20 * m))
    man.SetTopVolume(world)
    # facet: spherical shell cap intersected with a hexagonal prism
    mir_cut = TGeoPgon("mirCut", 0., 360., 6, 2)
    mir_cut.DefineSection(0, -100 * mm, 0, D / 2.)
    mir_cut.DefineSection(1, 100 * mm, 0, D / 2.)
    theta = math.degrees(math.asin(D / math.sqrt(3) / Rc))
    TGeoSphere("mirSphere", Rc, Rc + T, 180. - theta, 180.)
    TGeoTranslation("transZ", 0, 0, Rc).RegisterYourself()
    comp = TGeoCompositeShape("mirComposite", "mirSphere:transZ*mirCut")
    mirror = AMirror("mirror", comp)
    mirror.SetReflectance(0.85)
    cond = ABorderSurfaceCondition(world, mirror)
    cond.SetGaussianRoughness(roughness)
    for i, (x, y) in enumerate(_hex_lattice(D, n_facets)):
        r2 = x * x + y * y
        z = F - math.sqrt(F * F - r2)
        phi = math.degrees(math.atan2(y, x))
        rot = TGeoRotation(f"mirRot{i}", -phi + 90., 0, 0)
        th = math.degrees(math.atan2(math.sqrt(r2), 2 * F - z))
        rot2 = TGeoRotation("", phi - 90., th, 0)
        rot.MultiplyBy(rot2, False)
        # per-facet alignment error
        err = TGeoRotation("", 0, 0, 0)
        err.RotateX(math.degrees(tilt_sigma * rng.standard_normal()))
        err.RotateY(math.degrees(tilt_sigma * rng.standard_normal()))
        rot.MultiplyBy(err, True)
        world.AddNode(mirror, i + 1, TGeoCombiTrans(TGeoTranslation(x, y, z), rot))
    # focal plane 1.5 m across and an open-bottom camera box around it
    focal = AFocalSurface("focalPlane", TGeoTube("tubeCamera", 0, 75 * cm, 1 * mm))
    world.AddNode(focal, 1, TGeoTranslation(0, 0, F + 1 * mm))
    box_d, box_h, t = 1.7 * m, 1 * m, 10 * cm
    TGeoBBox("boxCamera", box_d / 2., box_d / 2., box_h / 2.)
    TGeoBBox("boxCamera2", box_d / 2. - t, box_d / 2. - t, box_h / 2. - t)
    TGeoTranslation("transZ1", 0, 0, F + box_h / 2.).RegisterYourself()
    TGeoTranslation("transZ2", 0, 0, F + box_h / 2. - t - 1 * mm).RegisterYourself()
    camera = AObscuration("cameraBox", TGeoCompositeShape("boxComposite", "boxCamera:transZ1-boxCamera2:transZ2"))
    world.AddNode(camera, 1)
    man.CloseGeometry()
    angles = np.linspace(0.0, max_angle, n_angles)
    batches = []
    for g, (a, n) in enumerate(zip(angles, _split(n_rays, n_angles))):
        r = a * deg
        tr = TGeoTranslation(-2 * F * math.sin(r), 0, 2 * F * math.cos(r))
        rot = TGeoRotation("", -90.0, a, 90.0)
        arr = ARayShooter.RandomCircle(400 * nm, 6.2 * m, n, rot, tr, (0.0, 0.0, -1.0), seed=seed * 1000 + g)
        b = _batch(arr, g)
        b["lam"] = np.random.default_rng(seed * 7919 + g).uniform(300 * nm, 600 * nm, n)
        batches.append(b)
    return man, _concat(batches)


# ---------------------------------------------------------------------------
# 4. light guide: 7x7 hexagonal Winston cones behind a window
# ---------------------------------------------------------------------------
SELLMEIER_WINDOW = (1.04, 0.23, 1.01, 0.0060, 0.020, 103.6)


def _light_guide_unit(world, tag, origin, r1, r2, window_index, reflectance, gap=1 * mm):
    """One 7x7 cone array + window, entrance plane at origin z."""
    cone = AGeoWinstonConePoly(f"cone{tag}", r1, r2, 6)
    dz = cone.GetDZ()
    pitch = 2 * r1
    # rows of 7 hexagons, alternate rows offset by half a pitch
    centres = [(pitch * (i + 0.5 * (j % 2)), pitch * (math.sqrt(3) / 2.0) * j) for i in range(7) for j in range(7)]
    cx = np.mean([c[0] for c in centres])
    cy = np.mean([c[1] for c in centres])
    centres = [(x - cx, y - cy) for x, y in centres]
    half = max(max(abs(x), abs(y)) for x, y in centres) + 2 * r1
    ox, oy, oz = origin
    block = AMirror(f"block{tag}", TGeoBBox(f"blockbox{tag}", half, half, dz))
    block.SetReflectance(reflectance)
    interior = AOpticalComponent(f"guide{tag}", cone)
    for k, (x, y) in enumerate(centres):
        block.AddNode(interior, k + 1, TGeoTranslation(x, y, 0))
    world.AddNode(block, 1, TGeoTranslation(ox, oy, oz - dz))
    window = ALens(f"window{tag}", TGeoBBox(f"windowbox{tag}", half, half, 0.25 * cm))
    window.SetRefractiveIndex(window_index)
    world.AddNode(window, 1, TGeoTranslation(ox, oy, oz + gap + 0.25 * cm))
    sensor = AFocalSurface(f"sensor{tag}", TGeoBBox(f"sensorbox{tag}", half, half, 0.05 * mm))
    world.AddNode(sensor, 1, TGeoTranslation(ox, oy, oz - 2 * dz - 0.05 * mm))
    return half


def light_guide(n_rays: int = 10_000_000, n_variants: int = 64, max_angle: float = 40.0, seed: int = 4):
    """64 variants of (entrance, exit) apothem around 25 mm / 12.5 mm, each a
    full 7x7 array + 5 mm window; the cone length follows from r1, r2
    (AGeoWinstonConePoly::SetWinstonDimensions)."""
    man = AOpticsManager("manager", "light guide")
    world = AOpticalComponent("world", TGeoBBox("worldbox", 20 * m, 20 * m, 5 * m))
    man.SetTopVolume(world)
    idx = ASellmeierFormula(*SELLMEIER_WINDOW)
    k = TGraph()
    for i, wl in enumerate((250 * nm, 700 * nm)):  # absorption length 1 m: k = lambda / (4 pi 100 cm)
        k.SetPoint(i, wl, ARefractiveIndex.AbsorptionLengthToExtinctionCoefficient(1 * m, wl))
    idx.SetExtinctionCoefficient(k)
    side = int(math.ceil(math.sqrt(n_variants)))
    spacing = 60 * cm
    rng = np.random.default_rng(seed)
    units = []
    for v in range(n_variants):
        r1 = 2.5 * cm * (1 + 0.1 * ((v % 8) - 3.5) / 3.5)
        r2 = 1.25 * cm * (1 + 0.1 * ((v // 8) - 3.5) / 3.5)
        origin = (spacing * (v % side - (side - 1) / 2), spacing * (v // side - (side - 1) / 2), 0.0)
        half = _light_guide_unit(world, v, origin, r1, r2, idx, 0.9)
        units.append((origin, half))
    man.CloseGeometry()
    batches = []
    for v, n in enumerate(_split(n_rays, n_variants)):
        (ox, oy, oz), half = units[v]
        gen = np.random.default_rng(seed * 100003 + v)
        th = np.radians(gen.uniform(0, max_angle, n))
        ph = gen.uniform(0, 2 * np.pi, n)
        d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), -np.cos(th)], axis=-1)
        # aim at a uniform point on the window top, start 3 cm above it
        tx = ox + gen.uniform(-0.9, 0.9, n) * half
        ty = oy + gen.uniform(-0.9, 0.9, n) * half
        tz = oz + 1 * mm + 0.5 * cm
        s = 3 * cm / np.cos(th)
        b = {"x": tx - s * d[:, 0], "y": ty - s * d[:, 1], "z": tz - s * d[:, 2], "dx": d[:, 0], "dy": d[:, 1],
             "dz": d[:, 2], "lam": gen.uniform(300 * nm, 600 * nm, n), "group": np.full(n, v, dtype=np.int32)}
        batches.append(b)
    return man, _concat(batches)


# ---------------------------------------------------------------------------
# 5. Schmidt-Cassegrain (tutorials/SchmidtCassegrain.C:39-110 prescription,
#    scaled from a 24-inch to a 2-m primary), 20-layer quarter-wave coating
# ---------------------------------------------------------------------------
LITHOSIL_Q = (0.670710810, 0.433322857, 0.877379057, 0.00449192312, 0.0132812976, 95.8899878)
INCH = 2.54 * cm


def _quarter_wave_stack(air, substrate, n_pairs=10, lam0=450 * nm, nh=2.4, nl=1.46):
    hi, lo = ARefractiveIndex(nh), ARefractiveIndex(nl)
    ml = AMultilayer(air, substrate)
    for _ in range(n_pairs):
        ml.InsertLayer(hi, lam0 / 4 / nh)
        ml.InsertLayer(lo, lam0 / 4 / nl)
    return ml


def _rot_of(tilt):
    """The secondary's drawn tilt as a matrix: RotateX then RotateY."""
    r = TGeoRotation("", 0, 0, 0)
    r.RotateX(math.degrees(tilt[0]))
    r.RotateY(math.degrees(tilt[1]))
    return r.R


def _sct_unit(world, tag, origin, corrector_index, coating, decenter=(0.0, 0.0), tilt=(0.0, 0.0),
              inc=(0.0, 0.0, 0.0, 0.0)):
    s = 100 * cm / (12.183 * INCH)  # 2-m primary
    off = 10 * cm
    ox, oy, oz = origin

    def tr(x, y, z):
        return TGeoTranslation(ox + x, oy + y, oz + z)

    # corrector: flat entrance, aspheric exit (polynomial in r^4.., scaled)
    c2 = -8.721454939626e-05 / INCH / s
    k = [0.0, 3.68090959e-7 / INCH ** 3 / s ** 3, 2.73643352e-11 / INCH ** 5 / s ** 5,
         3.20036892e-14 / INCH ** 7 / s ** 7]
    disk = AGeoAsphericDisk(f"corr{tag}", off * s, 0.0, (0.65 * INCH + off) * s, c2, 12 * INCH * s, 0.0)
    disk.SetPolynomials(0, [], 4, k)
    lens = ALens(f"corrector{tag}", disk)
    lens.SetRefractiveIndex(corrector_index)
    world.AddNode(lens, 1, tr(0, 0, 0))
    z_mid = 0.5 * (off * s + (0.65 * INCH + off) * s)
    half = 0.5 * 0.65 * INCH * s + 0.1 * mm
    ap = AObscuration(f"aperture{tag}", TGeoTube(f"aptube{tag}", 12 * INCH * s, 18 * INCH * s, half))
    world.AddNode(ap, 1, tr(0, 0, z_mid))
    # primary (concave, hole of 4 inch scaled)
    zp = ((0.65 + 40. + 32.) * INCH + off) * s
    cp = -1.049567394559e-002 / INCH / s
    pdisk = AGeoAsphericDisk(f"prim{tag}", zp, cp, zp + 0.1 * INCH * s, cp, 12.183 * INCH * s, 4 * INCH * s)
    pdisk.SetConicConstants(0.077235, 0.077235)
    primary = AMirror(f"primary{tag}", pdisk)
    world.AddNode(primary, 1, tr(0, 0, 0))
    # secondary (convex), with misalignment about its vertex
    zs = ((0.65 + 40. + 32. - 30.86635) * INCH + off) * s
    cs = -2.01270013787e-002 / INCH / s
    sdisk = AGeoAsphericDisk(f"sec{tag}", zs - 0.1 * INCH * s, cs, zs, cs, 4.322385947053 * INCH * s, 0)
    secondary = AMirror(f"secondary{tag}", sdisk)
    rot = TGeoRotation("", 0, 0, 0)
    rot.RotateX(math.degrees(tilt[0]))
    rot.RotateY(math.degrees(tilt[1]))
    c = np.array([0.0, 0.0, zs])
    t = c - rot.R @ c + np.array([decenter[0], decenter[1], 0.0]) + np.array([ox, oy, oz])
    if any(inc):
        # a further shift (inc[0], inc[1]) and rotation Rx(inc[2]) Ry(inc[3])
        # about the displaced vertex, axes of the world: the parameters the
        # adjoint differentiates (node shift / rotation at zero increment)
        ax, ay = inc[2], inc[3]
        rx = np.array([[1, 0, 0], [0, math.cos(ax), -math.sin(ax)], [0, math.sin(ax), math.cos(ax)]])
        ry = np.array([[math.cos(ay), 0, math.sin(ay)], [0, 1, 0], [-math.sin(ay), 0, math.cos(ay)]])
        ri = rx @ ry
        pivot = np.array([ox + decenter[0], oy + decenter[1], oz + zs])
        t = ri @ (t - pivot) + pivot + np.array([inc[0], inc[1], 0.0])
        rot = TGeoRotation("", 0, 0, 0)
        rot.SetMatrix(ri @ _rot_of(tilt))
    world.AddNode(secondary, 1, TGeoCombiTrans(t[0], t[1], t[2], rot))
    # focal screen behind the primary
    zf = ((0.65 + 40. + 32. - 30.86635 + 50.6706488) * INCH + off) * s
    screen = AFocalSurface(f"screen{tag}", TGeoBBox(f"screenbox{tag}", 5 * INCH * s, 5 * INCH * s, 5 * um))
    world.AddNode(screen, 1, tr(0, 0, zf + 5 * um))
    for mir in (primary, secondary):
        cond = ABorderSurfaceCondition(world, mir)
        cond.SetMultilayer(coating)
    return 12 * INCH * s, off * s


def schmidt_cassegrain(n_rays: int = 100_000_000, n_samples: int = 256, seed: int = 5,
                       decenter_sigma: float = 0.02 * cm, tilt_sigma: float = 0.1e-3, coating_table=None,
                       increments=None):
    """coating_table: None (per-ray CoherentTMMMixed of the stack), or the
    (lam_nbins, lam_min, lam_max, th_nbins, th_min, th_max) arguments of
    AMultilayer::PreCalculateCoherentTMM for the stack.  increments: None,
    or per sample (shift x, shift y, rotation x, rotation y) of its
    secondary on top of the drawn misalignment (_sct_unit)."""
    man = AOpticsManager("manager", "Schmidt-Cassegrain")
    man.DisableFresnelReflection(True)
    side = int(math.ceil(math.sqrt(n_samples)))
    spacing = 3.2 * m
    half_world = max(20 * m, spacing * side / 2 + 3 * m)
    world = AOpticalComponent("world", TGeoBBox("worldbox", half_world, half_world, 10 * m))
    man.SetTopVolume(world)
    air = ARefractiveIndex(1.0, 0.0)
    silica = ASellmeierFormula(*LITHOSIL_Q)
    coating = _quarter_wave_stack(air, silica)
    if coating_table is not None:
        coating.PreCalculateCoherentTMM(*coating_table)
    rng = np.random.default_rng(seed)
    units = []
    for v in range(n_samples):
        origin = (spacing * (v % side - (side - 1) / 2), spacing * (v // side - (side - 1) / 2), 0.0)
        dec = tuple(decenter_sigma * rng.standard_normal(2))
        tilt = tuple(tilt_sigma * rng.standard_normal(2))
        inc = tuple(increments[v]) if increments is not None else (0.0, 0.0, 0.0, 0.0)
        rap, zc = _sct_unit(world, v, origin, silica, coating, dec, tilt, inc)
        units.append((origin, rap, zc))
    man.CloseGeometry()
    batches = []
    for v, n in enumerate(_split(n_rays, n_samples)):
        (ox, oy, oz), rap, zc = units[v]
        tr = TGeoTranslation(ox, oy, oz + zc - 20 * cm)
        arr = ARayShooter.RandomCircle(450 * nm, rap * 0.98, n, None, tr, (0.0, 0.0, 1.0), seed=seed * 100003 + v)
        b = _batch(arr, v)
        b["lam"] = np.random.default_rng(seed * 7 + v).uniform(350 * nm, 650 * nm, n)
        batches.append(b)
    return man, _concat(batches)


CONFIGS = {
    "paraboloid": paraboloid,
    "davies_cotton": davies_cotton,
    "schwarzschild_couder": schwarzschild_couder,
    "light_guide": light_guide,
    "schmidt_cassegrain": schmidt_cassegrain,
}

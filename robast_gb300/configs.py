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

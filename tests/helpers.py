"""Scene builders shared by the tests (reference fixture makeTheWorld(),
tutorials/unittest_robast.py:47-55, and material scenes)."""
import json
import math
import os

import robast_gb300 as R

HERE = os.path.dirname(os.path.abspath(__file__))
m, cm, mm, um, nm = 100.0, 1.0, 0.1, 1e-4, 1e-7
deg = math.pi / 180.0


def make_the_world(limit=None):
    man = R.AOpticsManager("manager", "manager")
    world = R.AOpticalComponent("world", R.TGeoBBox("worldbox", 20 * m, 20 * m, 20 * m))
    man.SetTopVolume(world)
    if limit:
        man.SetLimit(limit)
    return man


def material(name):
    """Filmetrics table fixture (tests/golden/materials.json)."""
    with open(os.path.join(HERE, "golden", "materials.json")) as f:
        d = json.load(f)[name]
    idx = R.ARefractiveIndex()
    ng, kg = R.TGraph(), R.TGraph()
    for i, (w, n, k) in enumerate(zip(d["wavelength_nm"], d["n"], d["k"])):
        ng.SetPoint(i, w * nm, n)
        kg.SetPoint(i, w * nm, k)
    idx.SetRefractiveIndex(ng)
    idx.SetExtinctionCoefficient(kg)
    return idx


def glass_catalog():
    return R.AGlassCatalog(os.path.join(HERE, "golden", "glasses.agf"))


class MaterialScene:
    """A scene that registers refractive indices, multilayers and tables so
    that the oracle (and the GPU) can evaluate them by id."""

    def __init__(self, indices=(), multilayers=(), mirrors=()):
        self.man = make_the_world()
        world = self.man.GetTopVolume()
        self.lenses = []
        for i, idx in enumerate(indices):
            lens = R.ALens(f"lens{i}", R.TGeoBBox(f"lensbox{i}", 1, 1, 1))
            lens.SetRefractiveIndex(idx)
            world.AddNode(lens, 1, R.TGeoTranslation(0, 0, 10 * (i + 1)))
            self.lenses.append(lens)
        for j, ml in enumerate(multilayers):
            mir = R.AMirror(f"mlmirror{j}", R.TGeoBBox(f"mlbox{j}", 1, 1, 1))
            world.AddNode(mir, 1, R.TGeoTranslation(0, 0, -10 * (j + 1)))
            c = R.ABorderSurfaceCondition(world, mir)
            c.SetMultilayer(ml)
        self.mirrors = []
        for k, mir in enumerate(mirrors):
            world.AddNode(mir, 1, R.TGeoTranslation(10 * (k + 1), 0, 0))
            self.mirrors.append(mir)
        self.scene = self.man.CloseGeometry()
        b = self.scene.builder
        self.index_id = {id(i): b.index_ids[id(i)] for i in indices}
        self.ml_id = {id(ml): b.multilayer_ids[id(ml)] for ml in multilayers}
        self.volume_id = {id(v): b.volume_ids[id(v)] for v in mirrors}

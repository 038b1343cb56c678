"""GB300-native non-sequential ray tracing with ROBAST's API.

The hot path, AOpticsManager::TraceNonSequential over an ARayArray, runs as
hand-written sm_103a CUDA kernels behind the C ABI of include/robast_gb.h.
"""
from .geometry import (AGeoAsphericDisk, AGeoBezierPcon, AGeoBezierPgon, AGeoWinstonCone2D, AGeoWinstonConePoly,
                       TGeoBBox,
                       TGeoCombiTrans, TGeoCompositeShape, TGeoCone, TGeoHMatrix, TGeoMatrix, TGeoParaboloid, TGeoPcon, TGeoPgon, TGeoRotation,
                       TGeoShape, TGeoSphere, TGeoTranslation, TGeoTube, TGeoTubeSeg)
from .manager import AOpticsManager, ARay, ARayArray, ARayShooter, Scene
from .optics import (ABorderSurfaceCondition, ACauchyFormula, AFilmetrixDotCom, AFocalSurface, AGlassCatalog, ALens,
                     AMirror, AMixedRefractiveIndex, AMultilayer, AObscuration, AOpticalComponent, ARefractiveIndex,
                     ASchottFormula, ASellmeierFormula, TGeoVolume, TGraph, TGraph2D, TH2)

__all__ = [n for n in dir() if n[0].isupper()]

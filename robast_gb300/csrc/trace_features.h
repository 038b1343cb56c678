// trace_features.h -- optional scene features.  A tracer kernel instantiated
// without a feature compiles that code path out and is only launched on
// scenes that do not use it.
#pragma once

namespace rbg {
enum : unsigned {
  kFeatCSG = 1u,         // TGeo primitives other than boxes, composites
  kFeatWinston = 2u,     // AGeoWinstonConePoly
  kFeatLens = 4u,        // ALens volumes (refraction, bulk absorption)
  kFeatMultilayer = 8u,  // border conditions with thin films
  kFeatRough = 16u,      // roughness or Lambertian border conditions
  kFeatBVH = 32u,        // mothers with a BVH over their daughters
  kFeatAll = 63u
};
}  // namespace rbg

/*
 * robast_gb_layout.h -- canonical shape parameter layout of a flattened
 * scene (rbg_flat_scene.params).  rbg_scene_create() converts the user
 * layout of robast_gb.h into this one, adding the derived quantities that
 * the reference computes in its setters:
 *   AGeoAsphericDisk::SetAsphDimensions / SetConicConstants / ComputeBBox
 *     (src/AGeoAsphericDisk.cxx:971-1013, 164-243)
 *   AGeoWinstonConePoly::SetWinstonDimensions (src/AGeoWinstonConePoly.cxx:356-386)
 *   TGeoParaboloid coefficients z = a r^2 + b.
 * Angles stay in degrees (TGeo convention), lengths in cm.
 */
#ifndef ROBAST_GB_LAYOUT_H
#define ROBAST_GB_LAYOUT_H

/* BOX */
#define RBG_BOX_DX 0
#define RBG_BOX_DY 1
#define RBG_BOX_DZ 2
#define RBG_BOX_OX 3
#define RBG_BOX_OY 4
#define RBG_BOX_OZ 5
#define RBG_BOX_NP 6

/* TUBE (TGeoTube, TGeoTubeSeg): dphi >= 360 means a full tube */
#define RBG_TUBE_RMIN 0
#define RBG_TUBE_RMAX 1
#define RBG_TUBE_DZ 2
#define RBG_TUBE_PHI1 3
#define RBG_TUBE_DPHI 4
#define RBG_TUBE_NP 5

/* SPHERE (TGeoSphere) */
#define RBG_SPH_RMIN 0
#define RBG_SPH_RMAX 1
#define RBG_SPH_TH1 2
#define RBG_SPH_TH2 3
#define RBG_SPH_PHI1 4
#define RBG_SPH_DPHI 5
#define RBG_SPH_NP 6

/* PARABOLOID (TGeoParaboloid): solid = {|z| <= dz, a r^2 + b <= z} for a > 0
 * ({a r^2 + b >= z} for a < 0), a = 2 dz / (rhi^2 - rlo^2),
 * b = -dz - a rlo^2 */
#define RBG_PARA_RLO 0
#define RBG_PARA_RHI 1
#define RBG_PARA_DZ 2
#define RBG_PARA_A 3
#define RBG_PARA_B 4
#define RBG_PARA_NP 5

/* PGON: phi1 dphi nedges nz, z[nz], rmin[nz], rmax[nz] */
#define RBG_PGON_PHI1 0
#define RBG_PGON_DPHI 1
#define RBG_PGON_NEDGES 2
#define RBG_PGON_NZ 3
#define RBG_PGON_Z 4 /* z[i] = p[4+i], rmin[i] = p[4+nz+i], rmax[i] = p[4+2nz+i] */

/* PCON: phi1 dphi nz, z[nz], rmin[nz], rmax[nz] */
#define RBG_PCON_PHI1 0
#define RBG_PCON_DPHI 1
#define RBG_PCON_NZ 2
#define RBG_PCON_Z 3

/* ASPHERIC_DISK (AGeoAsphericDisk): surface 1 is the lower one (z1 < z2).
 * kappa = conic + 1.  origin_z / dz are fOrigin[2] / fDZ of ComputeBBox.
 * rseg = 1 when rmin > 0 (kGeoRSeg).  k1[npol1] then k2[npol2] follow. */
#define RBG_ASPH_Z1 0
#define RBG_ASPH_Z2 1
#define RBG_ASPH_C1 2
#define RBG_ASPH_C2 3
#define RBG_ASPH_KAPPA1 4
#define RBG_ASPH_KAPPA2 5
#define RBG_ASPH_RMIN 6
#define RBG_ASPH_RMAX 7
#define RBG_ASPH_NPOL1 8
#define RBG_ASPH_NPOL2 9
#define RBG_ASPH_ORIGIN_Z 10
#define RBG_ASPH_DZ 11
#define RBG_ASPH_RSEG 12
/* CalcF1/CalcF2 at rmin and rmax (the wall z ranges of DistToInner/Outer,
 * src/AGeoAsphericDisk.cxx:556-557,633-634); NaN where the sag is undefined */
#define RBG_ASPH_F1RMIN 13
#define RBG_ASPH_F2RMIN 14
#define RBG_ASPH_F1RMAX 15
#define RBG_ASPH_F2RMAX 16
#define RBG_ASPH_K 17
#define RBG_ASPH_MAXPOL 16

/* WINSTON_POLY (AGeoWinstonConePoly) and WINSTON_2D (AGeoWinstonCone2D,
 * stored with N = 2, DX = r1 and DY = the trough's half length) */
#define RBG_WIN_R1 0
#define RBG_WIN_R2 1
#define RBG_WIN_N 2
#define RBG_WIN_THETA 3
#define RBG_WIN_F 4
#define RBG_WIN_DZ 5
#define RBG_WIN_DX 6
#define RBG_WIN_DY 7
#define RBG_WIN_NP 8

/* COMPOSITE: left operand matrix (12) then right operand matrix (12) */
#define RBG_COMP_ML 0
#define RBG_COMP_MR 12
#define RBG_COMP_NP 24

/* Navigation constants (restated from TGeo / ROBAST):
 *  - RBG_BOUNDARY_PUSH: distance a boundary crossing moves past the surface
 *    (TGeoNavigator::FindNextBoundaryAndStep pushes the point by a small
 *    tolerance so that it is located in the next volume);
 *  - RBG_REFLECT_BACKSTEP: after a reflection the point steps back by
 *    kEpsilon = 1e-6 cm (src/AOpticsManager.cxx:20-21,241-243) plus the
 *    1e-6 cm that TGeoNavigator::Step adds to a geometric crossing step. */
#define RBG_BIG 1.0e30
#define RBG_BOUNDARY_PUSH 1.0e-9
#define RBG_REFLECT_BACKSTEP 2.0e-6
#define RBG_SPEED_OF_LIGHT_CM 2.99792458e10
/* bound on the rejection loops of the roughness sampler and on CSG crossing
 * lists; exceeding them sets RBG_ERR_CAP for the ray's trace call */
#define RBG_ROUGH_MAX_TRIES 1000
#define RBG_MAX_XINGS 48
/* deepest TGeoCompositeShape tree the flattener accepts (a composite of two
 * primitives has depth 1); the device walks deeper trees with explicit
 * stacks of this many frames plus one, so no kernel recurses */
#define RBG_MAX_COMPOSITE_DEPTH 6

#endif /* ROBAST_GB_LAYOUT_H */

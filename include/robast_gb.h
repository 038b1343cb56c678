/*
 * robast_gb.h -- C ABI of the GB300 non-sequential ray tracer.
 *
 * This is the drop-in boundary for ROBAST's hot path
 *   AOpticsManager::TraceNonSequential(ARayArray&)   (src/AOpticsManager.cxx:523-587)
 *   AOpticsManager::TraceNonSequential(TObjArray*)   (src/AOpticsManager.cxx:335-520)
 *   AOpticsManager::TraceNonSequential(ARay&)        (src/AOpticsManager.cxx:327-332)
 * declared at include/AOpticsManager.h:92-100.
 *
 * A caller (the C++ facade in robast_gb.hpp, the Python facade in the
 * robast_gb300 package, or a ROOT-side binding inside AOpticsManager) describes
 * the TGeo volume tree once as plain arrays (rbg_scene_desc), the library
 * flattens it into physical nodes with composed transforms, bounding boxes and
 * per-mother BVHs (rbg_scene), and rbg_trace() runs the whole per-ray state
 * machine on the GPU.  No torch types, no C++ types: plain pointers and sizes.
 *
 * Units follow ROBAST: length in cm (include/AOpticsManager.h:59-65), time in
 * s, wavelength in cm (400 nm = 4e-5), angles in rad unless a field says deg.
 */
#ifndef ROBAST_GB_H
#define ROBAST_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RBG_ABI_VERSION 2

/* ---- status codes (every entry point returns one) --------------------- */
enum {
  RBG_OK = 0,
  RBG_ERR_ARG = 1,         /* null pointer, negative size, bad option */
  RBG_ERR_SCENE = 2,       /* inconsistent scene description */
  RBG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  RBG_ERR_NAN = 4,         /* a ray had a NaN/zero direction or NaN origin */
  RBG_ERR_CAP = 5,         /* a bounded device loop hit its iteration cap */
  RBG_ERR_UNSUPPORTED = 6, /* feature outside this build (e.g. AGeo shape in CSG) */
  RBG_ERR_NOMEM = 7,       /* allocation failed */
  RBG_ERR_NODEVICE = 8,    /* no CUDA device visible */
  RBG_ERR_TOO_LARGE = 9    /* scene exceeds rbg_trace_noalloc's fixed array */
};

/* ---- per-ray fate: same values and order as ARay's private enum
 *      {kRun, kStop, kExit, kFocus, kSuspend, kAbsorb} (include/ARay.h:26) */
enum {
  RBG_RUN = 0,
  RBG_STOP = 1,
  RBG_EXIT = 2,
  RBG_FOCUS = 3,
  RBG_SUSPEND = 4,
  RBG_ABSORB = 5
};

/* ---- component kind = the C++ class of the TGeoVolume that the reference
 *      tests with IsA() (include/AOpticsManager.h:45-53,76-90) -------------- */
enum {
  RBG_KIND_LENS = 0,   /* ALens            */
  RBG_KIND_OBS = 1,    /* AObscuration     */
  RBG_KIND_MIRROR = 2, /* AMirror          */
  RBG_KIND_FOCUS = 3,  /* AFocalSurface    */
  RBG_KIND_OPT = 4,    /* AOpticalComponent */
  RBG_KIND_OTHER = 5   /* any other TGeoVolume */
};

/* ---- shapes ------------------------------------------------------------ */
enum {
  RBG_SHAPE_BOX = 1,            /* TGeoBBox                     */
  RBG_SHAPE_TUBE = 2,           /* TGeoTube / TGeoTubeSeg       */
  RBG_SHAPE_SPHERE = 3,         /* TGeoSphere                   */
  RBG_SHAPE_PARABOLOID = 4,     /* TGeoParaboloid               */
  RBG_SHAPE_PGON = 5,           /* TGeoPgon                     */
  RBG_SHAPE_PCON = 6,           /* TGeoPcon / TGeoCone(Seg)     */
  RBG_SHAPE_ASPHERIC_DISK = 7,  /* AGeoAsphericDisk             */
  RBG_SHAPE_WINSTON_POLY = 8,   /* AGeoWinstonConePoly          */
  RBG_SHAPE_COMPOSITE = 9,      /* TGeoCompositeShape node      */
  RBG_SHAPE_WINSTON_2D = 10     /* AGeoWinstonCone2D            */
};
enum { RBG_OP_UNION = 0, RBG_OP_INTERSECTION = 1, RBG_OP_SUBTRACTION = 2 };

/*
 * Shape parameters, in rbg_scene_desc.params starting at param_offset.
 * "User" layout (what a caller passes; mirrors each constructor):
 *   BOX            dx dy dz ox oy oz                    (half lengths, origin)
 *   TUBE           rmin rmax dz phi1 phi2               (deg; phi2-phi1>=360: full)
 *   SPHERE         rmin rmax theta1 theta2 phi1 phi2    (deg)
 *   PARABOLOID     rlo rhi dz
 *   PGON           phi1 dphi nedges nz  z[nz] rmin[nz] rmax[nz]   (deg; r = apothem)
 *   PCON           phi1 dphi nz  z[nz] rmin[nz] rmax[nz]           (deg)
 *   ASPHERIC_DISK  z1 curve1 z2 curve2 rmax rmin conic1 conic2 npol1 npol2
 *                  steps repeat  k1[npol1] k2[npol2]
 *   WINSTON_POLY   r1 r2 n
 *   WINSTON_2D     r1 r2 y                              (y: half length of the trough)
 *   COMPOSITE      (no params; op/left/right/left_matrix/right_matrix fields)
 * The flattened scene (rbg_flat_scene) holds a canonical layout that adds
 * derived quantities; it is documented in include/robast_gb_layout.h.
 */
typedef struct {
  int32_t type;
  int32_t param_offset;
  int32_t n_params;
  int32_t op;           /* composite only */
  int32_t left, right;  /* composite only: operand shape ids */
  int32_t left_matrix;  /* composite only: matrix id or -1 (identity) */
  int32_t right_matrix;
} rbg_shape_desc;

/* Tabulated functions (TGraph::Eval; TH2::Interpolate on a rectilinear grid).
 * 1D: params x[nx], y[nx].  2D: params x[nx], y[ny], z[nx*ny] with
 * z[ix*ny+iy]. */
enum { RBG_TABLE_1D = 1, RBG_TABLE_2D = 2 };
typedef struct {
  int32_t kind;
  int32_t nx, ny;
  int32_t param_offset;
} rbg_table_desc;

/* Refractive index models (include/ARefractiveIndex.h:25-68,
 * src/ASellmeierFormula.cxx:46-54, src/ACauchyFormula.cxx,
 * src/ASchottFormula.cxx, src/AMixedRefractiveIndex.cxx). k always comes from
 * k_table (-1: k = 0).  TABLE with n_table = -1 gives n = 1. */
enum {
  RBG_INDEX_TABLE = 1,
  RBG_INDEX_SELLMEIER = 2, /* coef: B1 B2 B3 C1 C2 C3 (um^2)          */
  RBG_INDEX_CAUCHY = 3,    /* coef: A B C  n = A + B/l^2 + C/l^4 (um) */
  RBG_INDEX_SCHOTT = 4,    /* coef: A0..A5                             */
  RBG_INDEX_MIXED = 5      /* mix_a, mix_b index ids, coef[0] = fraction of a */
};
typedef struct {
  int32_t kind;
  int32_t n_table, k_table;
  int32_t mix_a, mix_b;
  double coef[6];
} rbg_index_desc;

/* AMultilayer: layers[layer_offset .. layer_offset+n_layers), first = top
 * (incident) medium, last = bottom (substrate); their thickness is ignored
 * (semi-infinite) and they count as incoherent.  Per ray the tracer takes
 * CoherentTMMMixed (src/AMultilayer.cxx:240-481), or, after
 * PreCalculateCoherentTMM / PreCalculateIncoherentTMM
 * (include/AMultilayer.h:243-282), TH2::Interpolate of the tabulated
 * (lambda, theta) reflectance and transmittance: precalc = 1 tabulates the
 * coherent, 2 the incoherent (IncoherentTMM, :555-731) mixed-polarisation
 * values at the bin centres of lam_nbins x th_nbins bins over
 * [lam_min, lam_max) x [th_min, th_max) (lambda in cm, theta in rad). */
typedef struct {
  int32_t index;      /* refractive index id */
  int32_t coherent;
  double thickness;   /* cm */
} rbg_layer_desc;
typedef struct {
  int32_t layer_offset;
  int32_t n_layers;
  int32_t precalc;    /* 0 none, 1 coherent table, 2 incoherent table */
  int32_t lam_nbins, th_nbins;
  int32_t reserved;
  double lam_min, lam_max, th_min, th_max;
} rbg_multilayer_desc;

/* ABorderSurfaceCondition(component1, component2)
 * (include/ABorderSurfaceCondition.h:24-45).  component2 = -1 is a null
 * component (outside of the top volume). */
typedef struct {
  int32_t component1, component2;  /* volume ids */
  double sigma;                    /* Gaussian roughness (rad) */
  int32_t multilayer;              /* multilayer id or -1 */
  int32_t lambertian;
} rbg_border_desc;

/* A logical volume: TGeoVolume subclass + its optical properties. */
typedef struct {
  int32_t shape;
  int32_t kind;            /* RBG_KIND_* */
  double reflectance;      /* AMirror constant reflectance (default 1.0) */
  int32_t refl_table;      /* AMirror table: 1D in lambda or 2D in (lambda, angle); -1 none */
  int32_t index;           /* ALens refractive index id; -1: n = 1, k = 0 */
  int32_t qe_lambda_table; /* AFocalSurface QE(lambda); -1 none (QE = 1) */
  int32_t qe_angle_table;  /* AFocalSurface QE(angle);  -1 none */
} rbg_volume_desc;

/* TGeoVolume::AddNode / AddNodeOverlap */
typedef struct {
  int32_t mother;    /* volume id */
  int32_t daughter;  /* volume id */
  int32_t matrix;    /* matrix id (local -> mother) or -1 for identity */
  int32_t copy_no;
  int32_t overlap;
} rbg_placement_desc;

/* Scene description.  Matrices are 12 doubles each: a row-major 3x3 rotation
 * R followed by a translation t, master = R * local + t (TGeoMatrix
 * LocalToMaster convention). */
typedef struct {
  int32_t n_shapes;        const rbg_shape_desc* shapes;
  int32_t n_matrices;      const double* matrices;
  int32_t n_volumes;       const rbg_volume_desc* volumes;
  int32_t n_placements;    const rbg_placement_desc* placements;
  int32_t top_volume;
  int32_t n_tables;        const rbg_table_desc* tables;
  int32_t n_indices;       const rbg_index_desc* indices;
  int32_t n_layers;        const rbg_layer_desc* layers;
  int32_t n_multilayers;   const rbg_multilayer_desc* multilayers;
  int32_t n_borders;       const rbg_border_desc* borders;
  int64_t n_params;        const double* params;
} rbg_scene_desc;

/* ---- flattened scene (host view; what both the GPU tables and any CPU
 *      checker read) ------------------------------------------------------- */
typedef struct {
  int32_t parent;        /* physical node id of the mother; -1 for the top */
  int32_t volume;        /* logical volume id */
  int32_t shape;         /* = volumes[volume].shape, cached */
  int32_t kind;          /* = volumes[volume].kind, cached */
  int32_t child_begin;   /* into rbg_flat_scene.children */
  int32_t child_count;
  int32_t bvh_root;      /* into rbg_flat_scene.bvh, -1: scan children */
  int32_t depth;
  double m[12];          /* local -> master (global) */
  double lo[3], hi[3];   /* conservative master-frame bounding box */
} rbg_node;

/* Binary BVH over the children of one mother.  Leaves hold a range of
 * rbg_flat_scene.bvh_items (physical node ids).  Boxes are rounded outward
 * to float. */
typedef struct {
  float lo[3], hi[3];
  int32_t left;        /* internal: child index; leaf: -1 */
  int32_t right;       /* internal: child index; leaf: item count */
  int32_t item_begin;  /* leaf: first item */
  int32_t pad;
} rbg_bvh_node;

typedef struct {
  int32_t n_nodes;      const rbg_node* nodes;
  int32_t n_children;   const int32_t* children;
  int32_t n_bvh;        const rbg_bvh_node* bvh;
  int32_t n_bvh_items;  const int32_t* bvh_items;
  /* canonical copies of the description tables */
  int32_t n_shapes;     const rbg_shape_desc* shapes;
  int32_t n_volumes;    const rbg_volume_desc* volumes;
  int32_t n_tables;     const rbg_table_desc* tables;
  int32_t n_indices;    const rbg_index_desc* indices;
  int32_t n_layers;     const rbg_layer_desc* layers;
  int32_t n_multilayers; const rbg_multilayer_desc* multilayers;
  int32_t n_borders;    const rbg_border_desc* borders;
  int64_t n_params;     const double* params;   /* canonical layout */
  int32_t top_node;     /* always 0 */
} rbg_flat_scene;

typedef struct rbg_scene rbg_scene;

/* ---- rays ------------------------------------------------------------- */
/* Input rays, structure of arrays (ARay: last point x,y,z,t, direction,
 * lambda; src/ARay.cxx:28-36).  Directions are normalised on entry exactly
 * as ARay::SetDirection does (src/ARay.cxx:210-223). */
typedef struct {
  int64_t n;
  const double *x, *y, *z, *t;
  const double *dx, *dy, *dz;
  const double* lambda;
} rbg_rays;

/* Output, structure of arrays.  Any pointer may be NULL (not written).
 * npoints = ARay::GetNpoints() (the start point counts as one);
 * last_node = physical node id of the last ARay::AddNode (-1: a null node,
 * i.e. outside the top volume; -2: no node was ever added).
 * Optional history: hist_cap points per ray, hist_xyzt[(i*hist_cap+j)*4+k],
 * hist_node[i*hist_cap+j]; points past hist_cap are dropped, and the
 * slots past a ray's npoints hold node -3 and point (0, 0, 0, 0). */
typedef struct {
  uint8_t* status;
  int32_t* npoints;
  int32_t* last_node;
  double *x, *y, *z, *t;
  double *dx, *dy, *dz;
  int32_t hist_cap;
  double* hist_xyzt;
  int32_t* hist_node;
} rbg_result;

/* Trace options.  limit and disable_fresnel are AOpticsManager::SetLimit
 * (src/AOpticsManager.cxx:590-594, default 100) and
 * DisableFresnelReflection (include/AOpticsManager.h:73-75). */
enum {
  RBG_PREC_FP64 = 0,   /* plain FP64, one thread per ray */
  RBG_PREC_MIXED = 1   /* mixed precision wavefront tracer */
};
typedef struct {
  int32_t limit;
  int32_t disable_fresnel;
  uint64_t seed;          /* Philox key: every random draw is a function of
                             (seed, ray id, draw number) */
  uint64_t ray_id_offset; /* ray id of element 0 (for sharded/batched calls) */
  int32_t precision;      /* RBG_PREC_* */
  int32_t block_size;     /* threads per block.  FP64 tracer: up to 128
                             (0: 128).  Mixed tracer: 128 or 256 for the
                             lean instance (two-mirror telescopes; 0: the
                             scene's tuned value, rbg_scene_autotune, else
                             256); the other instances run at their own
                             measured size (256 for segmented reflectors,
                             128 otherwise).  Results do not depend on it. */
  /* mixed tracer: a warp refills its idle lanes with consecutive rays once
   * at least this many (1..32) are idle; 1 keeps every lane busy, 32 keeps
   * a warp's rays together (coherent paths).  0: the scene's tuned value
   * (rbg_scene_autotune), else the library default.  Results do not depend
   * on it. */
  int32_t compaction;
  /* the order in which the rays are taken up.
   * RBG_ORDER_SPATIAL (default) groups the rays by a cell of their
   * direction and, within it, of their start point, so the lanes of a warp
   * follow neighbouring paths; RBG_ORDER_INPUT takes them in input order.
   * Every ray keeps its index for its inputs, outputs and random draws:
   * results do not depend on it.  Both tracers honour it.  Batches under
   * 2^14 rays, batches beyond the scene's reserved workspace
   * (rbg_scene_reserve) without a workspace of their own (below), and
   * rbg_trace_noalloc use input order. */
  int32_t ray_order;
  /* Optional DEVICE workspace of the caller (256-byte aligned) for the
   * take-up order of rbg_trace: used when workspace_bytes >=
   * rbg_trace_workspace_bytes(n), otherwise the scene's reserved one is
   * (NULL / 0: the scene's).  It lets callers that rebuild scenes
   * (parameter scans, gradient steps) keep one buffer for all of them. */
  void* workspace;
  uint64_t workspace_bytes;
} rbg_trace_opts;

enum { RBG_ORDER_SPATIAL = 0, RBG_ORDER_INPUT = 1 };

/* ---- CORSIKA IACT photon bunches (ACorsikaIACTFile) ------------------- */
/* One photon bunch per element (struct bunch of CORSIKA's IACT option, as
 * ACorsikaIACTFile::ReadEvent stores it, src/ACorsikaIACTFile.cxx:443-455):
 * arrival position relative to the telescope (cm), emission height (cm),
 * arrival time (ns), direction cosines (cz = -sqrt(1 - cx^2 - cy^2)),
 * wavelength (nm, 0 = not set by CORSIKA) and photon count (fractional). */
typedef struct {
  int64_t n;
  int32_t *tel, *array;
  float *x, *y, *zem, *time, *cx, *cy, *cz, *lambda, *photons;
} rbg_bunches;

typedef struct rbg_corsika rbg_corsika;

/* ---- entry points ------------------------------------------------------ */
int rbg_abi_version(void);
const char* rbg_status_string(int status);
void rbg_trace_opts_default(rbg_trace_opts* opts);

/* Flatten a description (host only, no device work).  Replaces the scene
 * construction + TGeoManager::CloseGeometry() of the reference
 * (e.g. tutorials/SimpleParabolicTelescope.C:22-83). */
int rbg_scene_create(const rbg_scene_desc* desc, rbg_scene** out);
void rbg_scene_destroy(rbg_scene* scene);
int rbg_scene_flat(const rbg_scene* scene, rbg_flat_scene* out);
/* Copy the flattened tables to the current CUDA device (done lazily by
 * rbg_trace when needed). */
int rbg_scene_upload(rbg_scene* scene);
/* Make, on the current device, every device allocation the scene needs to
 * trace batches of up to max_rays rays: the scene tables (as
 * rbg_scene_upload), the take-up order workspace of rbg_trace, and the two
 * pipeline slots of rbg_trace_host for hist_cap history points per ray (no
 * counterpart in the reference, whose AOpticsManager allocates per ray on
 * the heap).  After it, rbg_trace allocates nothing; a reservation smaller
 * than an earlier one keeps the larger workspaces.  Waits for the device
 * when a workspace grows. */
int rbg_scene_reserve(rbg_scene* scene, int64_t max_rays, int32_t hist_cap);
/* Bytes of the take-up order workspace rbg_trace uses for n rays (0 for
 * batches it takes up in input order). */
size_t rbg_trace_workspace_bytes(int64_t n_rays);

/* AOpticsManager::TraceNonSequential over n rays whose buffers live in
 * DEVICE memory, on `stream` (a cudaStream_t, NULL = legacy default); the
 * call waits for the stream to read the trace's status back.  The per-ray
 * fates, points and directions land in `out`.  It allocates no device
 * memory: a scene not yet on the current device is uploaded first (as
 * rbg_scene_upload), and the spatial take-up order runs only when
 * rbg_scene_reserve sized its workspace for at least n rays (otherwise the
 * rays are taken up in input order, with the same results).  A scene's
 * queue head, error word and ray-order workspace serve one trace at a time:
 * traces of the same scene must not overlap (give each concurrent stream
 * its own scene). */
int rbg_trace(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
              const rbg_trace_opts* opts, void* stream);
/* rbg_trace without waiting: everything the trace does is put on `stream`
 * and the call returns; nothing is read back, allocated or synchronised,
 * so a host loop can run ahead and a CUDA graph can capture the call (the
 * tracer's whole batch then replays as one graph of the take-up order's
 * kernels and the persistent tracer).  The scene must already be on the
 * device (rbg_scene_reserve, or an earlier trace), and the workspace rule
 * is rbg_trace's.  No timing events are recorded.  rbg_trace_status reads
 * the status of the scene's last trace on `stream` (it waits for the
 * stream): RBG_OK, RBG_ERR_NAN or RBG_ERR_CAP, as rbg_trace returns. */
int rbg_trace_async(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
                    const rbg_trace_opts* opts, void* stream);
int rbg_trace_status(rbg_scene* scene, void* stream);

/* ACorsikaIACTFile::Open (src/ACorsikaIACTFile.cxx:191-257) on an
 * in-memory, decompressed eventio stream (the caller inflates .gz files):
 * reads the run header, the input card and the telescope positions.
 * RBG_ERR_ARG for a stream that is not a CORSIKA IACT file. */
int rbg_corsika_open(const uint8_t* data, int64_t nbytes, rbg_corsika** out);
void rbg_corsika_close(rbg_corsika* file);
/* The 273 words of the run header (ACorsikaIACTRunHeader, word 0 holds
 * the int32 tag) / of the current event's header (ACorsikaIACTEventHeader). */
int rbg_corsika_run_header(const rbg_corsika* file, float* out273);
int rbg_corsika_event_header(const rbg_corsika* file, float* out273);
/* The input card as newline-separated text (ACorsikaIACTFile::PrintInputCard);
 * returns the buffer size it needs. */
int rbg_corsika_input_lines(const rbg_corsika* file, char* buf, int64_t cap, int32_t* n_lines);
/* Telescope positions and radii, cm (GetTelescopeX/Y/Z/R). */
int rbg_corsika_telescopes(const rbg_corsika* file, int32_t cap, int32_t* n_tel, double* x, double* y,
                           double* z, double* r);
/* ACorsikaIACTFile::ReadEvent (:264-489): read forward to event `num`
 * (numbers start at 1); *event = num, or -1 when it is not found ahead.
 * RBG_ERR_ARG for a malformed block. */
int rbg_corsika_read_event(rbg_corsika* file, int32_t num, int32_t* event);
/* Array offsets of the current event (SetMultipleUseHeader). */
int rbg_corsika_offsets(const rbg_corsika* file, int32_t cap, int32_t* n_arrays, double* time_offset,
                        double* x, double* y);
/* Bunches of telescope `tel`, array `array` (< 0: any) of the current event
 * (the reference's TTree "tree"): count, and copy into host arrays of
 * capacity out->n (out->n becomes the count written). */
int64_t rbg_corsika_bunch_count(const rbg_corsika* file, int32_t tel, int32_t array);
int rbg_corsika_get_bunches(const rbg_corsika* file, int32_t tel, int32_t array, rbg_bunches* out);

/* ACorsikaIACTFile::GetRayArray (src/ACorsikaIACTFile.cxx:71-133) on the
 * GPU: every bunch in DEVICE arrays `b` becomes ceil(photons) rays (the
 * reference's `for (j = 0; j < photons; j++)`), started at height z (cm)
 * after back-projection along the bunch direction over
 * (z - tel_z) / |cz| (x, y and time; light speed c / refractive_index).
 * A bunch wavelength of 0 is drawn with 1/lambda uniform in
 * [1/lambda_max, 1/lambda_min] (nm) from Philox keyed by (seed, ray index);
 * the reference meant this law but passes its bunch-count limit as the
 * upper wavelength (:125).  Rays go to DEVICE arrays `out` of capacity
 * `capacity` (out->n is set); *n_rays receives the count.  With out == NULL
 * or too small a capacity only *n_rays is set (RBG_ERR_TOO_LARGE for the
 * latter).  At most 2^31 - 1 bunches per call, and a bunch counts at most
 * 2^32 rays.  `workspace` is a DEVICE buffer of
 * rbg_bunches_workspace_bytes(n) bytes; nothing is allocated.  Synchronises
 * `stream`. */
size_t rbg_bunches_workspace_bytes(int64_t n_bunches);
int rbg_bunches_to_rays(const rbg_bunches* b, double z, double tel_z, double refractive_index,
                        double lambda_min, double lambda_max, uint64_t seed, void* workspace,
                        rbg_rays* out, int64_t capacity, int64_t* n_rays, void* stream);

/* AMultilayer::CoherentTMM / IncoherentTMM / CoherentTMMMixed of a
 * multilayer of the scene for n (angle, wavelength) pairs in DEVICE arrays,
 * evaluated on the GPU in FP64 (the reference's multi-threaded vector
 * overloads, include/AMultilayer.h:157-237).  mode: 0 coherent, 1
 * incoherent, 2 what the tracer uses (the table when precalculated, else
 * coherent); pol: 0 s, 1 p, 2 mixed (s and p averaged).  The incidence
 * angle may be complex (th_im may be NULL).  Synchronises `stream`. */
int rbg_multilayer_rt(rbg_scene* scene, int32_t multilayer, int32_t mode, int32_t pol, int64_t n,
                      const double* th_re, const double* th_im, const double* lambda, double* R, double* T,
                      void* stream);

/* Autotuner of the mixed tracer (no counterpart in the reference, whose
 * thread split is fixed by the caller, src/AOpticsManager.cxx:529-567):
 * traces the DEVICE rays `in` with each candidate block size (256 and 128
 * where the scene runs the lean instance) and compaction threshold (1, 8,
 * 16, 32), two rounds each, keeps the fastest pair in the scene for later
 * calls that leave opts->block_size / opts->compaction at 0, and returns
 * the threshold in *chosen (rbg_scene_tuning reads both).  `out` receives
 * the trace results (identical for every candidate).  Synchronises
 * `stream`. */
int rbg_scene_autotune(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
                       const rbg_trace_opts* opts, void* stream, int32_t* chosen);
/* The mixed tracer's block size and compaction threshold for the scene:
 * rbg_scene_autotune's choice, else the defaults (block: 256 for scenes of
 * the lean instance, else the instance's own size; threshold 32).  Either
 * output pointer may be NULL. */
int rbg_scene_tuning(const rbg_scene* scene, int32_t* block_size, int32_t* compaction);
/* Set the scene's tuning directly (for instance an earlier process's
 * rbg_scene_autotune choice): block size 0 (default), 128 or 256;
 * compaction 0 (default) .. 32.  Results do not depend on either. */
int rbg_scene_set_tuning(rbg_scene* scene, int32_t block_size, int32_t compaction);

/* Same, with HOST buffers: copies the rays in, traces, copies the results
 * out and synchronises (the call a ROOT-side AOpticsManager binding makes,
 * src/AOpticsManager.cxx:523).  Its device staging (two pipeline slots of
 * up to 2^21 rays) is the scene's workspace: sized by rbg_scene_reserve, or
 * grown by the call itself when the reservation is smaller. */
int rbg_trace_host(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
                   const rbg_trace_opts* opts);

/* rbg_trace without any device allocation (no counterpart in the reference:
 * ROBAST traces on host threads).  For callers that cannot let a library
 * allocate or free device memory -- a real-time camera trigger or DAQ chain
 * or a serving process that owns all device memory in a fixed budget, where
 * cudaMalloc may fail and cudaFree would synchronise the whole device.  The
 * scene tables, the error word and the ray-queue counter live in one
 * statically allocated device array of 4 MiB (held by every GPU that loads
 * the library until exit); scenes whose flattened tables exceed it return
 * RBG_ERR_TOO_LARGE.  Buffers as rbg_trace (DEVICE rays and results); only
 * opts->precision == RBG_PREC_MIXED is accepted.  Calls share the array and
 * it keeps the last call's contents: calls that overlap on the GPU race.
 * Each call copies the scene tables in from host memory and waits for its
 * stream to read the error word back, so it cannot be captured into a CUDA
 * graph.  The first call on a device looks up the array's address with
 * that device current.  It sets no device limit: no tracer kernel recurses,
 * and the driver sizes each launch's stack to the kernel's static need. */
int rbg_trace_noalloc(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
                      const rbg_trace_opts* opts, void* stream);

/* Kernel timing (no counterpart in the reference): with on != 0, every
 * later rbg_trace of the scene records CUDA events on its stream around the
 * tracer kernel itself (not the take-up order's kernels), and
 * rbg_last_kernel_ms returns the last one's duration in ms (-1 when timing
 * is off).  For roofline measurements. */
int rbg_scene_set_timing(rbg_scene* scene, int32_t on);
double rbg_last_kernel_ms(const rbg_scene* scene);

/* Number of tracer kernel launches the last rbg_trace on this scene issued
 * (1 for either precision: the whole batch is one launch). */
int rbg_last_launch_count(const rbg_scene* scene);

/* ---- spot reductions ---------------------------------------------------- */
/* Focused-ray statistics per group (e.g. per field angle / variant) on
 * DEVICE arrays: sums[g*6 + k] accumulates (count, sum x, sum y, sum x^2,
 * sum y^2, sum t) over rays with status == RBG_FOCUS and group[i] == g
 * (group may be NULL: single group).  Used for the RMS spot size and the
 * effective area (tutorials/SchwarzschildCouder.C:133-161). */
int rbg_focal_moments(int64_t n, const uint8_t* status, const double* x,
                      const double* y, const double* t, const int32_t* group,
                      int32_t n_groups, double* sums, void* stream);

/* 2D histogram of focused rays on DEVICE arrays: counts[ix*ny+iy]
 * (TH2D::Fill semantics, under/overflow dropped). */
int rbg_focal_histogram(int64_t n, const uint8_t* status, const double* x,
                        const double* y, int32_t nx, double xlo, double xhi,
                        int32_t ny, double ylo, double yhi, double* counts,
                        void* stream);

/* AGeoUtil::ContainmentRadius (src/AGeoUtil.cxx:198-308) on a DEVICE
 * histogram counts[ix*ny+iy] with TH2 bin centres; r, x, y are host
 * outputs.  The whole search, its initial moments and every SumInRadius
 * probe (src/AGeoUtil.cxx:18-42) run on the GPU in one launch of one
 * thread-block cluster; nothing is allocated.  The call waits for
 * `stream`; concurrent calls are serialised.  RBG_ERR_CAP if the search
 * ran past 200000 histogram passes (never expected). */
int rbg_containment_radius(const double* counts, int32_t nx, double xlo,
                           double xhi, int32_t ny, double ylo, double yhi,
                           double fraction, double* r, double* x, double* y,
                           void* stream);
/* The same, stream-ordered: out (DEVICE, 4 doubles) receives r, x, y and a
 * status (0, or -1 for the pass cap); the call returns after the launch. */
int rbg_containment_radius_async(const double* counts, int32_t nx,
                                 double xlo, double xhi, int32_t ny,
                                 double ylo, double yhi, double fraction,
                                 double* out, void* stream);

/* ---- measurement -------------------------------------------------------- */
/* FP64 (bits = 64) or FP32 (bits = 32) fused multiply-add rate of the
 * current GPU in FLOP/s (2 per FMA), from a kernel of independent FMA
 * chains timed with CUDA events, best of two timed launches: the peak the
 * tracers' FP64-pipe and FP32-pipe roofline fractions are quoted against
 * (no counterpart in the reference).  Allocates and frees a small output
 * buffer; synchronises `stream`. */
int rbg_measure_fma_peak(int32_t bits, double* flops_per_s, void* stream);

/* Counted work of a mixed-precision trace (no counterpart in the reference):
 * the same trace as rbg_trace with RBG_PREC_MIXED, through a build of the
 * tracer that tallies each event of its arithmetic -- a boundary step, an
 * FP64 polish step of an aspheric root, a Horner term, an FP32 Newton
 * iteration, an FP32 screen, an FP64 fallback -- into counts[0 ..
 * rbg_event_kinds() - 1] (n_counts >= that).  rbg_event_flops gives the
 * FP64 and FP32 flops of one event of a kind, counted from the formulas it
 * evaluates (an FMA counts 2); the sum over kinds is the trace's algorithmic
 * flop count, the numerator of its FP64-pipe and FP32-pipe roofline
 * fractions.  Only scenes of boxes and aspheric disks (two-mirror
 * telescopes) are counted (RBG_ERR_UNSUPPORTED otherwise).  The take-up
 * order runs when opts lends a workspace.  Synchronises `stream`. */
int rbg_event_kinds(void);
int rbg_event_flops(int32_t kind, double* fp64, double* fp32);
int rbg_trace_count_events(rbg_scene* scene, const rbg_rays* in, rbg_result* out,
                           const rbg_trace_opts* opts, void* stream, uint64_t* counts,
                           int32_t n_counts);

/* ---- gradients ---------------------------------------------------------- */
/* Parameters the adjoint differentiates.  Shifts and rotations are small
 * rigid motions of a physical node applied in the master frame (the
 * derivative is taken at zero motion); coefficients are the polynomial
 * terms K_j of an AGeoAsphericDisk (SetPolynomials, src/AGeoAsphericDisk.cxx:
 * 1187-1204), on its lower (bit 0) and/or upper (bit 1) surface. */
enum {
  RBG_ADJ_ASPH_COEF = 1,   /* node, index = j, faces = bit mask */
  RBG_ADJ_NODE_SHIFT = 2,  /* node, index = master axis 0..2 */
  RBG_ADJ_NODE_ROTATE = 3  /* node, index = master axis 0..2, about pivot */
};
typedef struct {
  int32_t kind;
  int32_t node;
  int32_t index;
  int32_t faces;
  double pivot[3];
} rbg_adjoint_param;

/* Reverse-mode derivative of the final ray points (no counterpart in ROBAST,
 * which has no gradients: replaces the finite-difference Minuit scans of
 * tutorials/Optimize.C:60-205).  `fwd` is the DEVICE result of a trace of
 * the same rays with a point/node history (hist_cap >= the points of every
 * contributing ray); lambda (DEVICE, the rays' wavelengths) is needed when
 * the scene has lenses; dL_dx/dy/dz are DEVICE cotangents of each ray's
 * final point and g_points (DEVICE, n * hist_cap * 3, x y z per recorded
 * point) cotangents of its recorded reflection / refraction points (either
 * may be NULL = 0; a loss on a rim margin at a mirror uses the latter).
 * Accumulates (+=) into the DEVICE array dL_dparams:
 *   dL/dp_k = sum_i dL/dx_i . dx_i/dp_k
 * Segments are recomputed from the recorded hit points; surface
 * intersections (implicit-function rule at each hit), reflections (mirror
 * normal curvature included) and refractions (Snell's transmitted
 * direction, src/AOpticsManager.cxx:146-155, with the indices of the media
 * located along the path) are differentiated, with each ray's branches
 * (transmit, Fresnel or total internal reflection) held fixed.  Rays whose
 * path has more than 22 such events or an unsupported surface are skipped
 * and counted in *n_skipped (host, may be NULL). */
int rbg_trace_adjoint(rbg_scene* scene, int64_t n, const rbg_result* fwd,
                      const double* lambda, const double* dL_dx,
                      const double* dL_dy, const double* dL_dz,
                      const double* g_points, int32_t n_params,
                      const rbg_adjoint_param* params,
                      double* dL_dparams, int64_t* n_skipped, void* stream);

/* ---- ray sources -------------------------------------------------------- */
/* ARayShooter generators (include/ARayShooter.h:25-51,
 * src/ARayShooter.cxx:122-459) writing HOST arrays: the x, y, z, t, dx, dy,
 * dz and lambda arrays of `out` are written (their const is cast away) and
 * out->n is the capacity on entry, the number of rays written on return.
 * rot: row-major 3x3 (TGeoRotation, NULL = identity), tr: 3 (NULL = 0),
 * dir: local direction (NULL = (0, 0, 1)).  Draws are Philox(seed, first_id
 * + i) on a stream separate from the tracer's.
 * params:  CIRCLE rmax nr nphi | RANDOM_CIRCLE rmax | RANDOM_CONE r d |
 *          RANDOM_RECTANGLE dx dy | RANDOM_SPHERE - |
 *          RANDOM_SPHERICAL_CONE theta(deg) | RECTANGLE dx dy nx ny */
enum {
  RBG_SHOOT_CIRCLE = 1,
  RBG_SHOOT_RANDOM_CIRCLE = 2,
  RBG_SHOOT_RANDOM_CONE = 3,
  RBG_SHOOT_RANDOM_RECTANGLE = 4,
  RBG_SHOOT_RANDOM_SPHERE = 5,
  RBG_SHOOT_RANDOM_SPHERICAL_CONE = 6,
  RBG_SHOOT_RECTANGLE = 7
};
int rbg_shoot(int32_t kind, const double* params, int64_t n, const double* rot,
              const double* tr, const double* dir, uint64_t seed,
              uint64_t first_id, double lambda, rbg_rays* out);
/* The same generators writing DEVICE arrays on `stream` (one thread per
 * ray; params, rot, tr and dir stay host pointers): ray i draws exactly
 * what rbg_shoot draws for it, and the random-circle, -cone and -rectangle
 * sources and the grids give bit-identical rays (the sphere sources call
 * the device's cos / sin / acos, which may differ in the last bit).  out->n
 * is the capacity on entry and the count written on return; RBG_ERR_ARG if
 * the source needs more.  Returns after the launch; nothing is allocated. */
int rbg_shoot_device(int32_t kind, const double* params, int64_t n,
                     const double* rot, const double* tr, const double* dir,
                     uint64_t seed, uint64_t first_id, double lambda,
                     rbg_rays* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ROBAST_GB_H */

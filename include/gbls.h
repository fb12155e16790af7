/*
 * gbls.h -- C ABI of the GB300 narrow-band level-set advection library.
 *
 * This is the drop-in boundary for OpenVDB's level-set advection hot path:
 *   openvdb/openvdb/tools/LevelSetAdvect.h   class LevelSetAdvection   (:71-213)
 *   openvdb/openvdb/tools/LevelSetTracker.h  class LevelSetTracker     (:56-256)
 * Those are header-only C++ templates; a C++ caller keeps their call surface
 * through include/openvdb_gb300/LevelSetAdvect.h, which packs an OpenVDB
 * FloatGrid into a gbls_grid_desc and calls the functions below.  Every entry
 * point takes plain pointers and sizes, returns a gbls_status (0 = success)
 * and never throws; gbls_last_error() describes the last failure on the
 * calling thread.
 *
 * Numeric codes of schemes and trim modes equal the reference enums
 * (math/FiniteDifference.h:164-171 BiasedGradientScheme, :233-238
 * TemporalIntegrationScheme, tools/LevelSetTracker.h:45-50 TrimMode), so a
 * binding can pass the reference enum values straight through.
 */
#ifndef GBLS_H
#define GBLS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBLS_ABI_VERSION 4

/* ---- status codes ---------------------------------------------------- */
typedef enum gbls_status {
    GBLS_OK = 0,
    GBLS_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size                         */
    GBLS_ERR_VALUE = 2,            /* reference throws ValueError (bad scheme/map)  */
    GBLS_ERR_RUNTIME = 3,          /* reference throws RuntimeError (not a level set,
                                      non-uniform voxels)                           */
    GBLS_ERR_CUDA = 4,             /* a CUDA call failed                             */
    GBLS_ERR_OUT_OF_MEMORY = 5,
    GBLS_ERR_INTERRUPTED = 6,      /* the interrupter asked to stop                  */
    GBLS_ERR_DOMAIN = 7,           /* coordinates outside the supported index range */
    GBLS_ERR_UNSUPPORTED = 8,      /* input the device tree cannot represent         */
    GBLS_ERR_DEVICE_CHECK = 9      /* a device-side bounds check fired               */
} gbls_status;

/* ---- schemes (values equal the OpenVDB enums) ------------------------ */
enum {
    GBLS_FIRST_BIAS = 0,
    GBLS_SECOND_BIAS = 1,
    GBLS_THIRD_BIAS = 2,
    GBLS_WENO5_BIAS = 3,
    GBLS_HJWENO5_BIAS = 4
};
enum { GBLS_TVD_RK1 = 0, GBLS_TVD_RK2 = 1, GBLS_TVD_RK3 = 2 };
enum { GBLS_TRIM_NONE = 0, GBLS_TRIM_INTERIOR = 1, GBLS_TRIM_EXTERIOR = 2, GBLS_TRIM_ALL = 3 };

/* Arithmetic mode of the stencil kernels.
 * PARITY gives results bit-identical to the reference CPU path: every FP32
 *   operation in the reference's order without contraction, and the WENO5
 *   weights, which math/FiniteDifference.h:301-321 computes in FP64, as
 *   double-word FP32 pairs with an error bound that decides the reference's
 *   float result (the rare undecided evaluations run the FP64 formula).
 *   The environment variable GBLS_PARITY_FP64=1, read when a handle is
 *   created, selects kernels that evaluate every weight in FP64 instead
 *   (the same bits, slower; for cross-checking).
 * FAST evaluates everything in FP32 (contracted, shared sub-expressions). */
/* PARITY: bit-identical to the reference's FloatGrid path; FAST: FP32
 * arithmetic; FP64: the FloatGrid scheme (its constants as floats) with the
 * values and every value operation in double, the error oracle of the FP32
 * run.                                                                      */
enum { GBLS_MODE_PARITY = 0, GBLS_MODE_FAST = 1, GBLS_MODE_FP64 = 2 };

/* Transform kinds accepted (tools/LevelSetAdvect.h:257-276 accepts these four;
 * the device path supports the uniform-scale ones). */
enum {
    GBLS_MAP_UNIFORM_SCALE = 0,
    GBLS_MAP_UNIFORM_SCALE_TRANSLATE = 1,
    GBLS_MAP_TRANSLATION = 2
};

/* ---- host description of a FloatGrid level set -------------------------
 * The tree is OpenVDB's Tree4<float,5,4,3>: root -> 4096^3 upper internal
 * nodes (32^3 slots) -> 128^3 lower internal nodes (16^3 slots) -> 8^3 leaves.
 * Canonical order of every list is the reference's tree order (root map
 * order = lexicographic origin, then child offset), and tile tables hold 0.0f
 * at slots occupied by a child.  Tiles are inactive (level sets carry no
 * active tiles).  Leaf voxel n = (x<<6)|(y<<3)|z (tree/LeafNode.h:1069-1075);
 * mask word w holds voxels 64w..64w+63, bit b = voxel 64w+b.
 * Upper slot n = (x<<10)|(y<<5)|z with x=(i>>7)&31; lower slot n =
 * (x<<8)|(y<<4)|z with x=(i>>3)&15.                                          */
typedef struct gbls_grid_desc {
    double voxel_size;            /* uniform voxel size dx                      */
    double translation[3];        /* world offset of voxel (0,0,0)              */
    int32_t map_type;             /* GBLS_MAP_*                                 */
    float background;             /* outside value gamma > 0                    */
    int64_t leaf_count;
    int32_t* leaf_origins;        /* [leaf_count][3]                            */
    uint64_t* leaf_masks;         /* [leaf_count][8]                            */
    float* leaf_values;           /* [leaf_count][512]                          */
    int64_t lower_count;
    int32_t* lower_origins;       /* [lower_count][3]                           */
    float* lower_tiles;           /* [lower_count][4096]                        */
    int64_t upper_count;
    int32_t* upper_origins;       /* [upper_count][3]                           */
    float* upper_tiles;           /* [upper_count][32768]                       */
    int64_t root_tile_count;
    int32_t* root_tile_origins;   /* [root_tile_count][3]                       */
    float* root_tile_values;      /* [root_tile_count]                          */
} gbls_grid_desc;

/* Sizes of a grid (to allocate a gbls_grid_desc for gbls_download). */
typedef struct gbls_grid_counts {
    int64_t leaf_count;
    int64_t lower_count;
    int64_t upper_count;
    int64_t root_tile_count;
    int64_t active_voxel_count;
    float background;           /* current background (dilate / erode / resize change it) */
} gbls_grid_counts;

/* ---- velocity fields ----------------------------------------------------
 * The reference takes any functor with operator()(Coord ijk, float t)
 * (tools/LevelSetAdvect.h:32-52).  These kinds cover the callers of the path:
 *  CONSTANT     v(ijk,t) = constant  (DiscreteField of an empty Vec3fGrid whose
 *               background is `constant`, tools/VelocityFields.h:42-94)
 *  DENSE        aligned DiscreteField<Vec3fGrid>: the value stored at ijk inside
 *               [dense_origin, dense_origin+dense_dims), dense_background outside
 *  DEFORMATION  LeVeque's divergence-free deformation, see gbls_fields.h
 *  ROTATION     constant + omega x (ijk - center)
 *  HOST_SAMPLED any functor: the caller's host_sample(host_user, n, ijk, t,
 *               velocity) is called once per CFL substep, at the substep's
 *               start time t, with the index coordinates ijk[n][3] of the n
 *               active voxels in the reference's velocity order (leaves in
 *               tree order, voxels in offset order within a leaf), and fills
 *               velocity[n][3] (index-space units per time unit, as
 *               Advect::sampleField stores it, tools/LevelSetAdvect.h:
 *               426-493; the library negates it for backward advection and
 *               takes max|v|^2 from it).  The C++ drop-in passes every FieldT
 *               this way, calling field(ijk, t) or field(map(ijk), t) exactly
 *               as the reference's sample<Aligned> does.                     */
enum {
    GBLS_FIELD_CONSTANT = 0,
    GBLS_FIELD_DENSE = 1,
    GBLS_FIELD_DEFORMATION = 2,
    GBLS_FIELD_ROTATION = 3,
    GBLS_FIELD_HOST_SAMPLED = 4
};
typedef void (*gbls_host_sample_fn)(void* user, int64_t n, const int32_t* ijk, float t, float* velocity);

/* A level set's linear map, index -> world: x * scale + translation (scale 1
 * for a translation map, translation 0 for a uniform scale). */
typedef struct gbls_host_map {
    double scale;
    double translation[3];
} gbls_host_map;

/* A gbls_host_sample_fn for the reference's default velocity functor,
 * tools::EnrightField<float> (tools/VelocityFields.h:101-141): user points to
 * the level set's gbls_host_map; each voxel's world position goes through
 * the field's float formula with the C library's sinf / cosf, as the
 * reference evaluates it (tools/LevelSetAdvect.h:476-493).                  */
void gbls_host_sample_enright(void* user, int64_t n, const int32_t* ijk, float t, float* velocity);

typedef struct gbls_field_desc {
    int32_t kind;
    float constant[3];
    int32_t dense_origin[3];
    int32_t dense_dims[3];
    const float* dense_values;    /* [dims.x][dims.y][dims.z][3] in host memory  */
    float dense_background[3];
    float domain;                 /* DEFORMATION: voxels per unit length          */
    float period;                 /* DEFORMATION: T, in time units                */
    float scale;                  /* DEFORMATION: voxels per time unit per unit    */
    float omega[3];               /* ROTATION: angular velocity (rad / time unit)  */
    float center[3];              /* ROTATION: rotation centre (index space)       */
    /* DENSE: the velocity grid's own transform.  dense_map_type 0 = aligned
     * with the level set (the index-space lookup field(ijk)); otherwise
     * 1 + GBLS_MAP_*, with dense_voxel_size and dense_translation (world units):
     * each voxel samples the grid trilinearly (BoxSampler) at its world
     * position mapped into the grid's index space, as the reference's
     * non-aligned sample<false> path does (tools/LevelSetAdvect.h:476-486).  */
    int32_t dense_map_type;
    double dense_voxel_size;
    double dense_translation[3];
    gbls_host_sample_fn host_sample;   /* HOST_SAMPLED: the functor's sampler   */
    void* host_user;                   /* HOST_SAMPLED: its first argument      */
} gbls_field_desc;

typedef struct gbls_handle gbls_handle;   /* a device-resident level set      */
typedef struct gbls_field gbls_field;     /* a device-resident velocity field */

/* Interrupter hooks (util/NullInterrupter.h:29-49).  Any may be NULL.
 * was_interrupted returns non-zero to stop; the call then returns
 * GBLS_ERR_INTERRUPTED with the grid left at a substep boundary.            */
typedef struct gbls_interrupter {
    void (*start)(void* user, const char* name);
    void (*end)(void* user);
    int (*was_interrupted)(void* user, int percent);
    void* user;
} gbls_interrupter;

/* ---- library ----------------------------------------------------------- */
int gbls_abi_version(void);
const char* gbls_last_error(void);
/* Select the CUDA device used by handles created afterwards on this thread. */
int gbls_set_device(int device);

/* ---- grid lifetime (replaces the grid reference held by
 *      LevelSetTracker(GridT&) tools/LevelSetTracker.h:258-277) ---------- */
/* Upload a level set.  Returns GBLS_ERR_RUNTIME for a non-positive
 * background or voxel size (the reference requires GRID_LEVEL_SET class and
 * uniform voxels), GBLS_ERR_UNSUPPORTED for tiles other than +-background. */
int gbls_create(const gbls_grid_desc* desc, gbls_handle** out);
/* Replace the level set held by h with `desc` (the checks of gbls_create),
 * keeping h's device allocations, stream, precision mode, tracker state,
 * trimming and interrupter; the adjoint tape is discarded.  A long-lived
 * LevelSetAdvection / LevelSetTracker object re-uploads its grid this way on
 * every call.  After a refused upload h holds an empty level set.  Not for
 * batch handles.  No reference counterpart (the reference holds the grid).  */
int gbls_upload(gbls_handle* h, const gbls_grid_desc* desc);
int gbls_destroy(gbls_handle* h);
int gbls_get_counts(gbls_handle* h, gbls_grid_counts* out);
/* Copy the grid back in canonical order into caller-allocated arrays sized
 * by gbls_get_counts (replaces reading the mutated FloatGrid in place). */
int gbls_download(gbls_handle* h, gbls_grid_desc* out);
/* CUDA stream (cudaStream_t) for all work on this handle; NULL = default. */
int gbls_set_stream(gbls_handle* h, void* stream);

/* ---- tracker state (LevelSetTracker::State, tools/LevelSetTracker.h:74-83,
 *      setters :137-173) ------------------------------------------------- */
int gbls_set_tracker_state(gbls_handle* h, int spatial_scheme, int temporal_scheme,
                           int norm_count, int grain_size);
int gbls_get_tracker_state(gbls_handle* h, int* spatial_scheme, int* temporal_scheme,
                           int* norm_count, int* grain_size);
int gbls_set_trimming(gbls_handle* h, int trim_mode);       /* :171 */
int gbls_set_precision(gbls_handle* h, int mode);           /* GBLS_MODE_* */
/* GBLS_MODE_FP64 widens the level set's values to double (exactly); leaving
 * it rounds them back to FP32.  In FP64 mode gbls_advect and the tracker
 * operations run on double values with HJWENO5 (advection substeps in double
 * time, |v|^2 of the CFL limit in double at the first voxel holding the
 * maximum), gbls_download rounds to FP32 and gbls_get_active_values_f64
 * returns the doubles; batches, volumes, morphing, filters, the adjoint,
 * host-sampled fields and NanoVDB export are GBLS_ERR_UNSUPPORTED.          */
/* The active values in canonical order (leaf tree order, voxel order within
 * a leaf), as doubles, into host memory (FP32 level sets: widened).          */
int gbls_get_active_values_f64(gbls_handle* h, double* out);

/* ---- launch shapes (no reference counterpart) ------------------------------
 * The choices an autotuner makes per device and workload:
 *   stencil_min_ctas_rk / _norm  register budget of the PARITY RK-stage and
 *                                renormalisation kernels as the minimum
 *                                resident 64-thread CTAs per SM given to the
 *                                compiler: 0 (none: its heuristic, the
 *                                default), 1 (unconstrained), 14 or 16;
 *   cfl_leaves_per_block         leaves per CTA of the CFL maximum (8 threads
 *                                per leaf): 8, 16, 32 (default) or 64;
 *   rk_ctas_per_leaf             CTAs sharing one leaf in the PARITY RK stage
 *                                (each stages the leaf and takes every k-th
 *                                group of 64 active voxels): 1 (default), 2
 *                                or 4 -- more parallelism for small level sets.
 * Results do not depend on them.  gbls_time_launch_config times one RK stage,
 * one renormalisation stage and one CFL maximum of the current level set
 * under a configuration (reps launches after a warm-up, mean ms per launch
 * in ms[0..2]) and leaves the level set and the handle's configuration as
 * they were.                                                                 */
typedef struct gbls_launch_config {
    int32_t stencil_min_ctas_rk;
    int32_t stencil_min_ctas_norm;
    int32_t cfl_leaves_per_block;
    int32_t rk_ctas_per_leaf;
} gbls_launch_config;
int gbls_set_launch_config(gbls_handle* h, const gbls_launch_config* config);
int gbls_get_launch_config(gbls_handle* h, gbls_launch_config* config);
int gbls_time_launch_config(gbls_handle* h, const gbls_field* field, const gbls_launch_config* config,
                            int reps, float* ms);
int gbls_set_interrupter(gbls_handle* h, const gbls_interrupter* intr);

/* ---- LevelSetTracker operations ---------------------------------------- */
int gbls_track(gbls_handle* h);                              /* :302-315 */
int gbls_normalize(gbls_handle* h);                          /* :394-446 */
/* Replaces LevelSetTracker::normalize(const MaskT* mask) (tools/LevelSetTracker.h:
 * 94, 398-416; Normalizer :661-670): renormalise only the active voxels of the
 * mask leaves whose origins are leaves of the level set; the other active
 * voxels keep their values.  The mask is given as mask_leaf_count leaf origins
 * (xyz, multiples of 8) and 8 active-mask words per leaf (bit x<<6|y<<3|z).
 * GBLS_ERR_UNSUPPORTED when the mask covers a voxel that is inactive in the
 * level set (the reference would give that inactive voxel a value other than
 * +-background) or for a batch handle. */
int gbls_normalize_masked(gbls_handle* h, int64_t mask_leaf_count, const int32_t* mask_leaf_origins,
                          const uint64_t* mask_leaf_masks);
int gbls_prune(gbls_handle* h);                              /* :279-300 */
int gbls_dilate(gbls_handle* h, int iterations);             /* :317-337 */
int gbls_erode(gbls_handle* h, int iterations);              /* :339-349 */
int gbls_resize(gbls_handle* h, uint32_t half_width, int* changed); /* :351-364 */

/* ---- velocity fields ---------------------------------------------------- */
int gbls_field_create(const gbls_field_desc* desc, gbls_field** out);
int gbls_field_destroy(gbls_field* f);
/* New values for a DENSE field's grid from device memory [nx][ny][nz][3],
 * copied on `stream` (NULL: the default stream) before the call returns. */
int gbls_field_set_dense_device(gbls_field* f, const float* values, void* stream);

/* ---- LevelSetAdvection::advect (tools/LevelSetAdvect.h:216-418) ---------
 * Advects from t0 to t1 (t0 > t1 advects backward) with CFL-limited
 * substeps; each substep runs the temporal scheme's RK stages with the
 * biased spatial scheme, then the tracker pass.  cfl <= 0 selects the
 * reference constant {0.3,0.9,1.0}/sqrt(3) for RK1/2/3 (:459-461).
 * cfl > 0 imposes a CFL number the reference has no parameter for: the
 * result is that of the reference's advect(tau, tau') called on greedy
 * intervals tau' = tau + cfl*dx/max|v| (max|v| sampled at tau; the last
 * interval ends at t1), each with the reference's own substep loop.
 * *substeps receives the CFL count the reference returns (summed over the
 * intervals).                                                               */
int gbls_advect(gbls_handle* h, const gbls_field* field, int spatial_scheme,
                int temporal_scheme, float t0, float t1, float cfl, uint64_t* substeps);



/* ---- level-set filters ----------------------------------------------------------
 * Replaces tools::LevelSetFilter<FloatGrid> (tools/LevelSetFilter.h:93-157):
 * the filter followed by the tracker pass with h's tracker state.
 * LAPLACIAN, MEAN_CURVATURE, FILLET: one flow step; MEAN / GAUSSIAN: box
 * filter(s) and MEDIAN: median filter of half width `width` (1..3 on the
 * device, GBLS_ERR_UNSUPPORTED above); OFFSET: offset by `value` in
 * CFL-limited increments, each tracked.                                      */
enum {
    GBLS_FILTER_LAPLACIAN = 0,
    GBLS_FILTER_MEAN = 1,
    GBLS_FILTER_GAUSSIAN = 2,
    GBLS_FILTER_OFFSET = 3,
    GBLS_FILTER_MEAN_CURVATURE = 4,
    GBLS_FILTER_FILLET = 5,
    GBLS_FILTER_MEDIAN = 6
};
int gbls_filter(gbls_handle* h, int filter, int width, float value);
/* The same filter with an alpha mask: the `mask` argument of every filter of
 * tools::LevelSetFilter<FloatGrid, FloatGrid> (tools/LevelSetFilter.h:92-160)
 * with setMaskRange(mask_min, mask_max) (:77-83) and invertMask(invert_mask)
 * (:89).  alpha_mask is another single level set on the same device with the
 * same transform (looked up at each voxel's index; GBLS_ERR_UNSUPPORTED
 * otherwise); GBLS_ERR_VALUE unless mask_min < mask_max. */
int gbls_filter_masked(gbls_handle* h, int filter, int width, float value, gbls_handle* alpha_mask,
                       float mask_min, float mask_max, int invert_mask);

/* ---- level-set morphing ------------------------------------------------------
 * Replaces tools::LevelSetMorphing<FloatGrid>::advect (tools/LevelSetMorph.h:
 * 243-262): h moves towards the level set `target` with speed
 * phi - target (times the smooth-step of the alpha mask's value mapped from
 * [mask_min, mask_max] to [0, 1], or one minus it when invert_mask), CFL
 * substeps from t0 while t0 < t1, each followed by the tracker pass with h's
 * tracker state.  `target` and `alpha_mask` (may be NULL) are level sets
 * created with gbls_create on the same device with the same transform.
 * GBLS_ERR_VALUE for mask_min >= mask_max with a mask (setMaskRange).       */
int gbls_morph(gbls_handle* h, gbls_handle* target, gbls_handle* alpha_mask, int spatial_scheme,
               int temporal_scheme, float t0, float t1, float mask_min, float mask_max, int invert_mask,
               uint64_t* substeps);

/* ---- VolumeAdvection (tools/VolumeAdvect.h:76-560) ----------------------------
 * VolumeAdvection<Vec3fGrid, false>::advect<FloatGrid, Sampler<1, false>>(grid,
 * time_step) on the handle's grid (a FloatGrid volume such as a fog density:
 * inactive values +-background, tiles +-background, no active tiles), in
 * place: the grid is replaced by the advected copy, as the reference returns
 * it (dilated by ceil(max|v| dt / dx) voxels, sampled backwards along the
 * characteristics, limited, pruned).  `velocity` is the velocity grid: a
 * DENSE field (its own transform, or the volume's when dense_map_type is 0;
 * dense_background outside the box) or a CONSTANT one (a grid holding only
 * its background).  integrator: 0 SEMI, 1 MID, 2 RK3, 3 RK4, 4 MAC, 5 BFECC
 * (tools::Scheme::SemiLagrangian); limiter: 0 NO_LIMITER, 1 CLAMP, 2 REVERT
 * (the reference's default is CLAMP); substeps: setSubSteps (values below 1
 * count as 1).  max_velocity (may be NULL) receives getMaxVelocity().       */
int gbls_volume_advect(gbls_handle* h, const gbls_field* velocity, int integrator, int limiter, int substeps,
                       double time_step, double* max_velocity);
/* A handle for a general FloatGrid volume (the grid exchange of gbls_create
 * without its level-set checks: any background).  Such a handle takes
 * gbls_volume_advect, gbls_download and the counts; the level-set
 * operations return GBLS_ERR_UNSUPPORTED.                                    */
int gbls_create_volume(const gbls_grid_desc* desc, gbls_handle** out);

/* ---- adjoint ---------------------------------------------------------------
 * No counterpart in the reference (it has no derivatives).  While recording
 * is enabled, every CFL substep of gbls_advect (TVD_RK3 advection, TVD_RK1
 * tracker with normCount 1 and full trimming) is written to a tape on the
 * device.  gbls_adjoint_backward then runs the transposed substeps in reverse
 * with the recorded topology, upwind directions, Godunov branches and
 * trimming held fixed.  The substep lengths depend on the velocity (a
 * CFL-limited dt = CFL*dx/sqrt(max|v|^2) through the voxel holding the
 * maximum, the last substep of an interval through the ones before it, an
 * imposed CFL number's interval ends likewise), and dL/dv includes that
 * dependence.  Every sum runs in a fixed order: the results are
 * deterministic.
 *   dl_final[n_final]     dL/dphi on the active voxels after the last
 *                         recorded substep, in canonical order (tree-ordered
 *                         leaves, voxels in leaf order)
 *   dl_initial[n_initial] receives dL/dphi on the active voxels before the
 *                         first recorded substep, same order
 *   dl_velocity           receives dL/dv on a DENSE field's grid
 *                         [nx][ny][nz][3] (may be NULL; zero for other kinds)
 * `field` must be the field the recorded substeps used.  Recording again
 * discards the tape but keeps its device arrays for the new one (a
 * re-recorded forward pass of the same size allocates nothing); disabling
 * recording releases them.                                                  */
int gbls_adjoint_record(gbls_handle* h, int enable);
int gbls_adjoint_sizes(gbls_handle* h, int64_t* n_initial, int64_t* n_final, int64_t* substeps);
int gbls_adjoint_backward(gbls_handle* h, const gbls_field* field, const float* dl_final,
                          float* dl_initial, float* dl_velocity);
/* As gbls_adjoint_backward, but dL/dv (dense field layout) is ADDED into
 * dl_velocity_device, device memory of the handle's device, and nothing of it
 * is copied to the host: a checkpointed reverse sweep accumulates the
 * velocity gradient of its segments in place.  No reference counterpart.    */
int gbls_adjoint_backward_accumulate(gbls_handle* h, const gbls_field* field, const float* dl_final,
                                     float* dl_initial, float* dl_velocity_device);
/* As gbls_adjoint_backward_accumulate with dl_final and dl_initial in device
 * memory as well (dL/dv ADDED into dl_velocity_device, which may be NULL):
 * the device-resident path of a torch.autograd.Function.  No reference
 * counterpart.                                                               */
int gbls_adjoint_backward_device(gbls_handle* h, const gbls_field* field, const float* dl_final,
                                 float* dl_initial, float* dl_velocity_device);
/* The active values of the level set in canonical order (tree-ordered
 * leaves, voxels in leaf order) to / from device memory of the handle's
 * device, on the handle's stream; setting them refreshes the sign mask and
 * leaves the topology unchanged.  No reference counterpart (the reference
 * edits values through tree accessors).                                     */
int gbls_get_active_values_device(gbls_handle* h, float* out);
int gbls_set_active_values_device(gbls_handle* h, const float* in);

/* ---- batches of independent level sets --------------------------------------
 * A batch handle holds n level sets (instances) that share the voxel size and
 * background; gbls_batch_advect advances every instance i from t0 to t1 with
 * its own CFL substep sequence exactly as n separate
 * LevelSetAdvection::advect calls would (tools/LevelSetAdvect.h:338-418),
 * in one set of kernel launches per substep.  fields[i] is instance i's
 * velocity (CONSTANT, DEFORMATION or ROTATION); substeps[i] receives its CFL
 * count.  At most 512 instances.  The tracker state and the precision mode
 * of the handle apply to every instance.                                      */
#define GBLS_MAX_INSTANCES 512
int gbls_batch_create(int32_t n, const gbls_grid_desc* descs, gbls_handle** out);
int gbls_batch_instances(gbls_handle* h, int32_t* n);
int gbls_batch_get_counts(gbls_handle* h, int32_t instance, gbls_grid_counts* out);
int gbls_batch_download(gbls_handle* h, int32_t instance, gbls_grid_desc* out);
int gbls_batch_advect(gbls_handle* h, const gbls_field_desc* fields, int spatial, int temporal,
                      float t0, float t1, float cfl, uint64_t* substeps);

/* ---- measurement ----------------------------------------------------------
 * Counters since the last gbls_reset_stats.  voxel_updates is the sum over
 * CFL substeps of the active voxel count at the start of the substep.  With
 * profiling enabled the stencil kernels are bracketed by CUDA events on the
 * handle's stream and their device time and algorithmic bytes (FP32 values
 * read and written for active voxels only) are accumulated.               */
typedef struct gbls_stats {
    uint64_t substeps;
    uint64_t voxel_updates;
    uint64_t kernel_launches;      /* every kernel this library launched    */
    uint64_t rk_launches;          /* advection RK stage kernel             */
    uint64_t norm_launches;        /* renormalise / trim kernel             */
    double rk_ms, norm_ms;         /* device time (profiling only)          */
    double rk_bytes, norm_bytes;   /* algorithmic bytes of those launches   */
    uint64_t dilated_voxels;       /* voxels renormalised by track passes   */
    int64_t active_voxels;         /* current                               */
    int64_t leaves;                /* current                               */
} gbls_stats;
int gbls_get_stats(gbls_handle* h, gbls_stats* out);
int gbls_reset_stats(gbls_handle* h);
int gbls_set_profiling(gbls_handle* h, int enable);

/* ---- allocation-free active-voxel count ----------------------------------
 * No counterpart in the reference (its trees live in host memory).
 * Returns in *out the same count as gbls_get_counts' active_voxel_count, but
 * allocates no device memory: for host applications that give the library a
 * fixed device-memory budget and forbid allocations afterwards.  Scratch is a
 * 512 KiB static device array (at most 2,097,152 leaves; larger grids are
 * rejected with GBLS_ERR_INVALID_ARGUMENT; the environment variable
 * GBLS_NOALLOC_MAX_LEAVES can lower that limit).  Every call looks up the
 * array's device address on the handle's device.  Calls that overlap on the
 * GPU share the array and race.                                             */
int gbls_count_active_noalloc(gbls_handle* h, int64_t* out);

/* ---- host construction of level sets ------------------------------------
 * gbls_host_sphere replaces tools::createLevelSetSphere
 * (tools/LevelSetSphere.h:219-230): same rasterisation, background and
 * signed flood fill, so the result equals the reference grid voxel for voxel.
 * gbls_host_union_of_spheres rasterises the union of spheres directly (the
 * minimum of the sphere distances, then the same signed flood fill).
 * gbls_host_grid_view returns a descriptor pointing into the host grid's
 * arrays (valid until gbls_host_grid_free).                                 */
typedef struct gbls_host_grid gbls_host_grid;
int gbls_host_sphere(float radius, const float center[3], float voxel_size, float half_width,
                     gbls_host_grid** out);
int gbls_host_union_of_spheres(int64_t n, const float* centers, const float* radii,
                               float voxel_size, float half_width, gbls_host_grid** out);
/* A torus around the y axis (no counterpart in OpenVDB; batch fixtures). */
int gbls_host_torus(float major_radius, float minor_radius, const float center[3],
                    float voxel_size, float half_width, gbls_host_grid** out);
int gbls_host_grid_view(gbls_host_grid* g, gbls_grid_desc* view);
/* math::WENO5<float> (math/FiniteDifference.h:301-321) by the double-word
 * evaluation that the PARITY kernels run on the FP32 pipes, on n operand
 * quintuples v[5i..5i+4]: decided[i] = 1 when out[i] is the reference's
 * float, 0 when the kernels would evaluate the FP64 formula instead.     */
int gbls_host_weno5_exact(int64_t n, const float* v, float* out, uint8_t* decided);
/* The sign of that result where the three candidate sums of WENO5 agree,
 * which lets the PARITY renormalisation skip derivatives that
 * GodunovsNormSqrd clamps to zero: sign[i] = +1 (result >= 0), -1
 * (result <= 0), 2 (five zero operands: the result is a zero) or 0
 * (undecided).                                                             */
int gbls_host_weno5_sign(int64_t n, const float* v, int8_t* sign);
/* The same certificate for the backward operands d[6i..6i+4] (sb[i]) and
 * the forward operands d[6i+5], d[6i+4], ..., d[6i+1] (sf[i]) of n lines
 * of six differences at once, as the renormalisation evaluates it.         */
int gbls_host_weno5_sign_pair(int64_t n, const float* d, int8_t* sb, int8_t* sf);
/* The same WENO5 on the device, as the PARITY kernels evaluate it (the
 * double-word evaluation, the FP64 formula where it leaves the rounding
 * undecided): out[i] for the quintuple v[5i..5i+4]; decided[i] = 1 where
 * the double-word evaluation decided (decided may be NULL).  v, out and
 * decided are device arrays; runs on `stream` (NULL: the default stream)
 * and returns when done.                                                   */
int gbls_weno5_exact_device(const float* v, int64_t n, float* out, uint8_t* decided, void* stream);
int gbls_host_grid_free(gbls_host_grid* g);
const char* gbls_host_last_error(void);

/* ---- .vdb files (host) ----------------------------------------------------
 * OpenVDB's file format 225 for level-set FloatGrids (Tree_float_5_4_3),
 * read and written on the host; errors through gbls_host_last_error.
 * gbls_vdb_write replaces io::File::write (io/File.h:130, the stream layout
 * of io/Archive.cc:1010-1080 and 1261-1450): `count` grids from exchange
 * descriptors (tree order), named `names[i]` (NULL or "" allowed; unique
 * names are made as io::Archive::write makes them), with the grid class
 * "level set" and the statistics metadata io::Archive adds
 * (file_bbox_min/max, file_voxel_count, file_compression), data compressed
 * with COMPRESS_ACTIVE_MASK only (readable by every OpenVDB build).
 * gbls_vdb_grid_count / gbls_vdb_grid_info list the grids (io::File::
 * getGrids / readAllGridMetadata, io/File.h:107-150): unique name, grid type
 * (with a "_HalfFloat" suffix for half-float storage) and class, written as
 * NUL-terminated strings truncated to the given capacities.
 * gbls_vdb_read replaces io::File::readGrid (io/File.h:150): the grid named
 * `name` (unique name first, then grid name), or the `index`-th grid when
 * `name` is NULL, as a host grid for gbls_host_grid_view / gbls_upload.
 * GBLS_ERR_RUNTIME: not a VDB file, truncated or corrupt, non-uniform scale
 * (the tracker's RuntimeError); GBLS_ERR_INVALID_ARGUMENT: no such grid;
 * GBLS_ERR_UNSUPPORTED: another grid type, active tiles, Blosc/zlib data,
 * instanced trees, rotated transforms, format versions before 222.         */
int gbls_vdb_write(const char* path, int32_t count, const gbls_grid_desc* grids,
                   const char* const* names);
int gbls_vdb_grid_count(const char* path, int32_t* count);
int gbls_vdb_grid_info(const char* path, int32_t index, char* name, int64_t name_cap,
                       char* grid_type, int64_t type_cap, char* grid_class, int64_t class_cap);
int gbls_vdb_read(const char* path, const char* name, int32_t index, gbls_host_grid** out);

/* ---- NanoVDB export (host) -------------------------------------------------
 * Replaces nanovdb::tools::createNanoGrid(openvdb::FloatGrid, StatsMode,
 * CheckMode) (nanovdb/tools/CreateNanoGrid.h:162-168): the NanoGrid<float>
 * buffer (NanoVDB 32.9, breadth-first) of a level set in the exchange
 * layout, byte for byte what the reference writes.  stats_mode: 0 Disable,
 * 1 BBox, 2 MinMax, 3 All (node statistics combined in tree order);
 * checksum_mode: 0 Disable, 1 Partial (CRC-32 of the grid and tree headers),
 * 2 Full (also the blocked CRC-32 of the nodes).
 * With out == NULL only *size is set; otherwise out_capacity must be at least
 * the size.  Errors through gbls_host_last_error: GBLS_ERR_UNSUPPORTED for
 * names of 256 characters or more.                                          */
int gbls_nanovdb_export(const gbls_grid_desc* desc, const char* name, int32_t stats_mode,
                        int32_t checksum_mode, uint8_t* out, int64_t out_capacity, int64_t* size);
/* NanoVDB index grid: createNanoGrid<FloatGrid, ValueOnIndex>(grid, channels,
 * includeStats, includeTiles) (CreateNanoGrid.h:184-190): nodes hold offsets
 * into a value array (background first, four statistics slots per node when
 * both flags are set, active values per leaf), leaves their 9-bit prefix
 * sums; with channels = 1 the value array follows as blind data
 * "channel_0".  Byte for byte the reference's buffer, except the alignment
 * padding after the channel, which the reference leaves uninitialised.
 * channels > 1 is GBLS_ERR_UNSUPPORTED: the reference copies channel i from
 * (its start - value count), across that padding.                          */
/* NanoGrid<float> buffer -> host grid in the exchange layout (the
 * direction of nanovdb::tools::nanoToOpenVDB, nanovdb/tools/NanoToOpenVDB.h),
 * for gbls_host_grid_view / gbls_create.  GBLS_ERR_UNSUPPORTED for other value
 * types, active tiles and rotated maps; GBLS_ERR_RUNTIME for a non-NanoVDB or
 * truncated buffer.                                                          */
int gbls_nanovdb_import(const uint8_t* buffer, int64_t size, gbls_host_grid** out);
int gbls_nanovdb_export_index(const gbls_grid_desc* desc, const char* name, int32_t channels,
                              int32_t include_stats, int32_t include_tiles, int32_t checksum_mode,
                              uint8_t* out, int64_t out_capacity, int64_t* size);

/* ---- NanoVDB on the device ---------------------------------------------------
 * The same buffers written on the device straight from a handle's device
 * tree, byte for byte what gbls_nanovdb_export / gbls_nanovdb_export_index
 * write for the downloaded grid (and so what the reference's createNanoGrid
 * writes, nanovdb/tools/CreateNanoGrid.h:162-190): the advected level set
 * goes to NanoVDB's device consumers (ReadAccessor, the ValueOnIndex decode
 * of nanovdb/NanoVDB.h:4144-4170, samplers, ray marchers) without a host
 * round trip.  `instance` is -1 for a level-set handle, else the batch
 * instance.  `out` is device memory, 32-byte aligned (cudaMalloc), at least
 * *size bytes; with out == NULL only *size is set.  Runs on the handle's
 * stream and returns with the buffer complete.                              */
int gbls_nanovdb_export_device(gbls_handle* h, int32_t instance, const char* name, int32_t stats_mode,
                               int32_t checksum_mode, void* out, int64_t out_capacity, int64_t* size);
int gbls_nanovdb_export_index_device(gbls_handle* h, int32_t instance, const char* name, int32_t channels,
                                     int32_t include_stats, int32_t include_tiles, int32_t checksum_mode,
                                     void* out, int64_t out_capacity, int64_t* size);
/* A level-set handle from a NanoGrid<float> buffer in device memory (or host
 * memory): the tree is walked through its links as gbls_nanovdb_import
 * walks it, the internal nodes are read on the host and the leaves gathered
 * on the device.  A device buffer must be 32-byte aligned.  Errors as
 * gbls_nanovdb_import and gbls_create.                                       */
int gbls_create_from_nanovdb(const void* buffer, int64_t size, gbls_handle** out);
/* A device consumer of those buffers: nanovdb::ReadAccessor::getValue and
 * isActive (nanovdb/NanoVDB.h) at n index coordinates ijk[3i..3i+2], for a
 * NanoGrid<float> (values) or a NanoGrid<ValueOnIndex> (indices into its
 * value array: the LeafData<ValueOnIndex>::getValue decode,
 * nanovdb/NanoVDB.h:4144-4170).  grid, ijk and the outputs are device
 * arrays (active may be NULL); runs on `stream` (NULL: the default stream)
 * and returns when done.  Every read is bounds-checked against `size`:
 * GBLS_ERR_RUNTIME for a truncated or corrupt buffer.                      */
int gbls_nanovdb_probe(const void* grid, int64_t size, const int32_t* ijk, int64_t n, float* values,
                       uint64_t* indices, uint8_t* active, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBLS_H */

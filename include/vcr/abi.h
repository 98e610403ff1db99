/*
 * vcr — GB300-native volumetric cloud light-transport core: the C-ABI.
 *
 * Every entry point is `extern "C"`, takes plain pointers, sizes and POD
 * structs, and returns a vcr_status.  No exception crosses this boundary and
 * no CUDA or C++ type appears in a signature: streams are passed as `void*`
 * (a cudaStream_t, 0 = the legacy default stream).
 *
 * Conventions
 *  - A vcr_ctx owns all device memory it allocates (grid bricks, accumulation
 *    images, photon maps, beams, BVH nodes, network weights, scratch).
 *  - Host structs are copied at the call; the caller keeps ownership.
 *  - Calls are stream-ordered and asynchronous unless documented otherwise;
 *    calls on one context must come from one host thread at a time (the
 *    reference also records and submits from a single thread, main.cpp:603-712).
 *  - Device-side waits are bounded; a wait that runs out reports
 *    VCR_ERR_TIMEOUT instead of hanging.
 *  - vcr_last_error(ctx) returns a human-readable message for the last
 *    failing call on that context (NULL ctx: the last creation failure).
 *
 * The reference drives its GLSL compute shaders through the RenderTechnique
 * interface (CloudRendering-Vulkan/RenderTechnique.h:15-67); each group of
 * entry points below names the reference call it replaces.
 */
#ifndef VCR_ABI_H
#define VCR_ABI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define VCR_API __declspec(dllexport)
#else
#define VCR_API __attribute__((visibility("default")))
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                             */
/* ------------------------------------------------------------------------ */
typedef enum vcr_status {
  VCR_OK = 0,
  VCR_ERR_INVALID = 1,     /* bad argument (null pointer, size, enum)        */
  VCR_ERR_CUDA = 2,        /* a CUDA runtime call failed                     */
  VCR_ERR_OOM = 3,         /* device allocation failed                      */
  VCR_ERR_TIMEOUT = 4,     /* a bounded device-side wait ran out             */
  VCR_ERR_STATE = 5,       /* call out of order (e.g. pass before a grid)    */
  VCR_ERR_IO = 6,          /* file could not be read or written              */
  VCR_ERR_UNSUPPORTED = 7, /* feature or size not supported                  */
  VCR_ERR_CAPACITY = 8     /* an output buffer was too small (data dropped)  */
} vcr_status;

typedef struct vcr_ctx vcr_ctx;

/* ------------------------------------------------------------------------ */
/* Enums                                                                    */
/* ------------------------------------------------------------------------ */
typedef enum vcr_precision {
  VCR_PREC_FP32 = 0,
  VCR_PREC_FP16 = 1, /* FP16 texels, FP32 scale per 8^3 brick */
  VCR_PREC_BF16 = 2  /* BF16 texels, FP32 scale per 8^3 brick */
} vcr_precision;

typedef enum vcr_rng_mode {
  VCR_RNG_PCG = 0,     /* counter-keyed PCG stream per (seed, path, pass)    */
  VCR_RNG_XORSHIFT = 1 /* the shaders' xorshift32 (PathTracer.comp:220-241)  */
} vcr_rng_mode;

typedef enum vcr_nee_mode {
  VCR_NEE_RATIO = 0,       /* unbiased ratio tracking toward the sun          */
  VCR_NEE_SHADOW_VOLUME = 1 /* shadow-volume lookup (PathTracer.comp:406-411) */
} vcr_nee_mode;

typedef enum vcr_sky_mode {
  VCR_SKY_CONSTANT = 0, /* constant radiance vcr_params.sky                 */
  VCR_SKY_GRADIENT = 1  /* five-stop gradient (PathTracer.comp:104-113)      */
} vcr_sky_mode;

typedef enum vcr_tracker {
  VCR_TRACKER_GLOBAL = 0, /* one global majorant (PathTracer.comp:318-361)    */
  VCR_TRACKER_DDA = 1     /* per-brick majorants walked by a 3D DDA           */
} vcr_tracker;

typedef enum vcr_buffer_id {
  VCR_BUF_IMAGE_MEAN = 0,   /* float32 RGB, W*H*3: accumulated mean          */
  VCR_BUF_IMAGE_SUM = 1,    /* float64 RGB, W*H*3: raw FP64 sums             */
  VCR_BUF_PATH_STATS = 2,   /* uint32 x4 per pixel of the last pass          */
  VCR_BUF_PPM_STATS = 3,    /* float64 x4 per pixel: N, R, flux(luminance)   */
  VCR_BUF_SHADOW_VOLUME = 4 /* float32 n^3 shadow-volume texels              */
} vcr_buffer_id;

/* ------------------------------------------------------------------------ */
/* POD restatements of the reference's uniform blocks                       */
/* ------------------------------------------------------------------------ */

/* Device selection (the reference picks one Vulkan queue,
 * VulkanPhysicalDevice.cpp:102-104). */
typedef struct vcr_device_desc {
  int32_t device;  /* CUDA device ordinal */
  uint32_t flags;  /* reserved, 0 */
} vcr_device_desc;

/* Grid3D<float> header (Grid3D.h:9-41): voxel counts and voxel size. */
typedef struct vcr_grid_desc {
  uint32_t size[3];
  uint32_t _pad;
  double voxel_size[3];
} vcr_grid_desc;

/* CloudProperties (UniformBuffers.h:71-78).  max_extinction is the
 * density majorant; vcr_grid_upload/vcr_grid_generate set it to
 * max(grid max, 0.01) as SetCloudProperties does (main.cpp:152). */
typedef struct vcr_cloud {
  float bounds_min[3];
  float bounds_max[3];
  float max_extinction;
  float base_scaling;
  float density_scaling;
} vcr_cloud;

/* CameraProperties (UniformBuffers.h:15-69).  Image width = 2*half_width. */
typedef struct vcr_camera {
  float position[3];
  float forward[3];
  float right[3];
  float up[3];
  float near_plane;
  float pixel_size_x;
  float pixel_size_y;
  int32_t half_width;
  int32_t half_height;
} vcr_camera;

/* Parameters (UniformBuffers.h:80-112) plus the light and the semantic
 * switches.  The phase_* terms follow Parameters::SetPhaseG; use
 * vcr_params_set_phase_g to fill them. */
typedef struct vcr_params {
  uint32_t max_events;     /* scatter events per path; 0 = until escape      */
  float light_intensity;   /* sun irradiance (Parameters.lightIntensity)     */
  float phase_g;
  float phase_one_plus_g2;
  float phase_one_minus_g2;
  float phase_one_over_2g;
  int32_t isotropic;
  float albedo;            /* single-scattering albedo (1 = reference PT)    */
  float sun_dir[3];        /* unit direction the sunlight travels            */
  float sky[3];            /* constant sky radiance (VCR_SKY_CONSTANT)       */
  uint32_t sky_mode;       /* vcr_sky_mode                                   */
  uint32_t rng_mode;       /* vcr_rng_mode                                   */
  uint32_t nee_mode;       /* vcr_nee_mode                                   */
  uint32_t tracker;        /* vcr_tracker                                    */
  uint32_t nrc_events;     /* >0: terminate into the radiance cache after    */
                           /*     this many events (vcr_nrc_*)               */
} vcr_params;

/* ShadowVolumeProperties (UniformBuffers.h:114-167), derived state included
 * (bounds, basis, voxel size); vcr_shadow_volume_setup fills it. */
typedef struct vcr_shadow_volume {
  float bounds_min[3];
  float bounds_max[3];
  float light_dir[3];
  float right[3];
  float up[3];
  float basis_change[9]; /* row-major 3x3 world -> (right, up, light) */
  uint32_t voxel_axis_count;
  float voxel_size;
} vcr_shadow_volume;

/* Performance knobs of the DDA wavefront tracker (no reference counterpart;
 * the reference uses one global majorant, PathTracer.comp:338).
 * majorant_level selects DDA cells of (8 << level) voxels per axis, 0..3;
 * it changes how random numbers are consumed (not the expected image), so
 * it is part of a render's determinism key.  fast_math changes results
 * (within the floating-point rounding of the functions it swaps); the other
 * fields change only the schedule, never a result bit. */
typedef struct vcr_tuning {
  uint32_t majorant_level;  /* 0..3 */
  uint32_t dda_steps;       /* majorant cells a lane may walk per wavefront step, >= 1 */
  uint32_t stage_majorants; /* 1: stage the level's majorants in shared memory (TMA bulk copy) when they fit */
  uint32_t block_threads;   /* wavefront CTA size: 128 or 256 */
  uint32_t corner_blocks;   /* 1 (default): density lookups read a per-cell block of the 8 decoded trilinear
                               corners (32 bytes, one sector) built from the bricks, 32 B per voxel of device
                               memory; 0: they gather the 8 texels from the bricks (switching it off frees the
                               blocks).  Same values either way. */
  uint32_t fast_math;       /* 0 (default): the tracker's device arithmetic is the oracle's, operation for
                               operation (no contracted multiply-adds, the library's own log / exp / sincos
                               series), so images are bit-exact with it.  1: a second build of the same kernel
                               with contracted FMAs and the hardware log / exp / sincos approximations; a
                               path's decisions can then differ from the oracle's where a random number falls
                               within rounding of a threshold.  The autotuner keeps the caller's choice. */
} vcr_tuning;

/* PushConstants (UniformBuffers.h:6-13) for one progressive pass. */
typedef struct vcr_pass_desc {
  uint32_t seed;       /* render seed                                         */
  uint32_t pass_index; /* 0-based pass; the RNG key and the running mean use it */
  uint32_t spp;        /* camera samples per pixel in this pass (>=1)          */
  uint32_t crop[4];    /* x0, y0, w, h; w == 0 renders the whole frame         */
  uint32_t flags;      /* VCR_PASS_* */
} vcr_pass_desc;

#define VCR_PASS_RECORD_STATS 1u /* write VCR_BUF_PATH_STATS for this pass    */
#define VCR_PASS_NO_ACCUMULATE 2u /* overwrite instead of adding to the sums  */

/* Seeded Perlin-fBm density generator (the synthetic stand-in for the
 * reference's cloud files, models/mycloud.xyz). */
typedef struct vcr_fbm_desc {
  uint64_t seed;
  uint32_t octaves;
  float lacunarity;
  float gain;
  float base_frequency; /* noise frequency over the longest grid axis */
} vcr_fbm_desc;

/* ------------------------------------------------------------------------ */
/* Context lifecycle                                                        */
/* Replaces: RenderTechnique construction + VulkanDevice (main.cpp:765-840) */
/* ------------------------------------------------------------------------ */
VCR_API vcr_status vcr_create(vcr_ctx** out, const vcr_device_desc* desc);
VCR_API vcr_status vcr_destroy(vcr_ctx* ctx);
VCR_API const char* vcr_last_error(const vcr_ctx* ctx);
VCR_API uint32_t vcr_version(void);
/* Blocks until all work the context queued has finished (vkDeviceWaitIdle,
 * main.cpp:269); also reports any device-side error word. */
VCR_API vcr_status vcr_synchronize(vcr_ctx* ctx);

/* Limits of the device-side waits (the reference waits without a limit,
 * vkWaitForFences with UINT64_MAX, main.cpp:606).  sort_lookback: polls of
 * a predecessor tile's look-back word before a radix-sort tile gives up
 * (default 1<<22); stage_wait: mbarrier polls for the copy that stages a
 * majorant level in shared memory (default 1<<24).  A wait that runs out
 * sets the device error word, which vcr_synchronize (or, for the
 * allocation-free sort, vcr_sort_noalloc_status) reports as
 * VCR_ERR_TIMEOUT; a sort whose wait ran out has an unspecified order (it
 * stays inside its output buffers), a pass whose staging wait ran out reads
 * the majorants from global memory and renders the same image.  The limits
 * are process-wide and apply to launches queued after the call; NULL
 * restores the defaults.  Small limits exist to test the timeout path. */
typedef struct vcr_wait_limits {
  uint32_t sort_lookback;
  uint32_t stage_wait;
} vcr_wait_limits;
VCR_API vcr_status vcr_set_wait_limits(const vcr_wait_limits* limits);
VCR_API vcr_status vcr_get_wait_limits(vcr_wait_limits* out);

/* ------------------------------------------------------------------------ */
/* Host-side helpers for the reference's parameter structs                 */
/* ------------------------------------------------------------------------ */
/* Parameters::SetPhaseG (UniformBuffers.h:93-106): clamps g to +-0.95. */
VCR_API vcr_status vcr_params_set_phase_g(vcr_params* p, float g);
/* SetCloudProperties (main.cpp:145-163): bounds from voxel size x count x
 * base scaling, x/y centred, z from 0. */
VCR_API vcr_status vcr_cloud_from_grid(const vcr_grid_desc* grid, float base_scaling,
                                       float density_scaling, vcr_cloud* out);
/* CameraProperties defaults + SetResolution/SetFOV (UniformBuffers.h:15-58). */
VCR_API vcr_status vcr_camera_look(vcr_camera* cam, const float position[3],
                                   const float forward[3], float fov_y_deg,
                                   float near_plane, int32_t width, int32_t height);
/* ShadowVolumeProperties::SetLightDirection + SetOrigin
 * (UniformBuffers.h:131-166) for a cloud AABB. */
VCR_API vcr_status vcr_shadow_volume_setup(vcr_shadow_volume* sv, const float light_dir[3],
                                           const float bounds_min[3], const float bounds_max[3],
                                           uint32_t voxel_axis_count);

/* ------------------------------------------------------------------------ */
/* Density grid                                                             */
/* Replaces: Grid3D<float> load + UpdateCloudData upload (main.cpp:266-335)
 *           + QueueUpdateCloudData/QueueUpdateCloudDataSampler             */
/* ------------------------------------------------------------------------ */
/* Upload an x-fastest float grid (Grid3D memory order, Grid3D.h:116) from
 * host memory, brick it at `precision`, build the brick majorant grid.
 * Synchronous with respect to the host buffer (it may be reused on return). */
VCR_API vcr_status vcr_grid_upload(vcr_ctx* ctx, const vcr_grid_desc* desc,
                                   const float* host_density, vcr_precision precision);
/* Same, generating the density on the device from a seeded fBm. */
VCR_API vcr_status vcr_grid_generate(vcr_ctx* ctx, const vcr_grid_desc* desc,
                                     const vcr_fbm_desc* fbm, vcr_precision precision);
/* Global density maximum of the stored grid (Grid3D::GetMajorant,
 * Grid3D.h:180-192) and brick-grid dimensions. */
VCR_API vcr_status vcr_grid_info(vcr_ctx* ctx, float* out_max_density,
                                 uint32_t out_bricks[3]);
/* Read one level of the majorant pyramid (float per cell, x-fastest).
 * Level 0 has one cell per 8^3 brick: the max decoded texel over the brick
 * plus a one-texel halo; level l+1 takes the max over 2x2x2 cells of level
 * l; level l has ceil(bricks / 2^l) cells per axis. */
VCR_API vcr_status vcr_grid_read_majorants(vcr_ctx* ctx, uint32_t level, float* host_out, size_t count);
/* The stored grid decoded to dense floats (what the trackers sample: FP16 /
 * BF16 texels times their brick's scale), x fastest, count = X*Y*Z; out is
 * host or device memory.  Synchronous. */
VCR_API vcr_status vcr_grid_read_dense(vcr_ctx* ctx, float* out, size_t count);
/* Densities at n world positions (device pointers; float3 in, float out),
 * through the same trilinear fetch the trackers use. */
VCR_API vcr_status vcr_grid_sample(vcr_ctx* ctx, const float* d_pos, float* d_out,
                                   uint32_t n, void* stream);

/* .xyz file I/O (Grid3D::Load Grid3D.h:44-90, GridData::save GridData.h:14-25).
 * The file stores z fastest; memory is x fastest.  Pass a NULL data pointer
 * to vcr_xyz_read to query the header only. */
VCR_API vcr_status vcr_xyz_read(const char* path, vcr_grid_desc* desc, float* host_out,
                                size_t capacity);
VCR_API vcr_status vcr_xyz_write(const char* path, const vcr_grid_desc* desc,
                                 const float* host_data);
/* The fBm generator on the host (same float arithmetic as the device one). */
VCR_API vcr_status vcr_fbm_fill_host(const vcr_grid_desc* desc, const vcr_fbm_desc* fbm,
                                     float* host_out);

/* ------------------------------------------------------------------------ */
/* Scene state (QueueUpdateCameraProperties / QueueUpdateParameters /       */
/* QueueUpdateShadowVolume + UpdateDescriptorSets)                          */
/* ------------------------------------------------------------------------ */
VCR_API vcr_status vcr_set_cloud(vcr_ctx* ctx, const vcr_cloud* cloud);
VCR_API vcr_status vcr_set_camera(vcr_ctx* ctx, const vcr_camera* cam);
VCR_API vcr_status vcr_set_params(vcr_ctx* ctx, const vcr_params* params);
/* SetFrameReferences (RenderTechniquePT.cpp:63-80): a headless FP64 RGB
 * accumulation target of width x height; clears the running sums. */
VCR_API vcr_status vcr_set_frame(vcr_ctx* ctx, uint32_t width, uint32_t height);
/* Zero the running sums (frameCount = 1 reset, main.cpp:262). */
VCR_API vcr_status vcr_reset_accumulation(vcr_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* Shadow volume (RenderTechniqueSV::RecordDrawCommands,                    */
/* RenderTechniqueSV.cpp:102-113 + ShadowVolume.comp:77-93)                  */
/* ------------------------------------------------------------------------ */
VCR_API vcr_status vcr_shadow_volume_build(vcr_ctx* ctx, const vcr_shadow_volume* sv,
                                           void* stream);

/* ------------------------------------------------------------------------ */
/* Path tracing (RenderTechniquePT::RecordDrawCommands,                     */
/* RenderTechniquePT.cpp:129-168 + PathTracer.comp:366-425)                  */
/* ------------------------------------------------------------------------ */
/* One progressive pass: `spp` camera paths per pixel of the crop, added to
 * the FP64 sums.  vcr_params.tracker selects the reference per-pixel
 * global-majorant tracker or the persistent DDA wavefront tracker. */
VCR_API vcr_status vcr_pt_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
/* `count` consecutive progressive passes (first->pass_index, +1, ...) of the
 * DDA wavefront tracker in one launch: the same paths, random streams and
 * per-pass radiance as `count` calls of vcr_pt_pass (the FP64 sums equal
 * up to the order of their additions).  One persistent launch lets the
 * lanes that would idle while a pass's longest paths finish run the next
 * pass's paths.  Needs the DDA tracker; with the radiance cache
 * (nrc_events > 0) the paths of all `count` passes end in the same weights
 * and the cache's query capacity must hold count x crop x spp queries.  No
 * VCR_PASS_RECORD_STATS or VCR_PASS_NO_ACCUMULATE.  vcr_pt_counters then
 * reports the totals of all `count` passes.  Replaces `count` frames of
 * RenderTechniquePT::RecordDrawCommands (RenderTechniquePT.cpp:129-168)
 * whose images are not displayed in between. */
VCR_API vcr_status vcr_pt_passes(vcr_ctx* ctx, const vcr_pass_desc* first, uint32_t count, void* stream);
/* Tracker tuning (vcr_tuning).  Defaults: level 2, 4 steps, staging on,
 * 256 threads.  vcr_autotune_pt times one pass of `pass` per candidate on
 * `stream` (the passes are rendered into the sums and then reset), keeps
 * the fastest and returns it. */
VCR_API vcr_status vcr_set_tuning(vcr_ctx* ctx, const vcr_tuning* t);
VCR_API vcr_status vcr_get_tuning(vcr_ctx* ctx, vcr_tuning* out);
VCR_API vcr_status vcr_autotune_pt(vcr_ctx* ctx, const vcr_pass_desc* pass, vcr_tuning* out, void* stream);
/* Counters of the last vcr_pt_pass: [0] paths, [1] density lookups,
 * [2] scatter events, [3] DDA cell visits. */
VCR_API vcr_status vcr_pt_counters(vcr_ctx* ctx, uint64_t out[4]);

/* Trace the majorant-grid DDA of n rays (device float3 origins and unit
 * directions, already inside or entering the cloud box).  For ray i, up to
 * max_cells visits are written at out_cells[i*max_cells ..] as (linear cell
 * index) and out_t[2*(i*max_cells+k) ..] as (t_enter, t_exit); out_count[i]
 * gets the number of visits.  Bit-exact against the CPU oracle. */
VCR_API vcr_status vcr_dda_trace(vcr_ctx* ctx, const float* d_origin, const float* d_dir,
                                 uint32_t n, uint32_t max_cells, uint32_t* d_out_cells,
                                 float* d_out_t, uint32_t* d_out_count, void* stream);

/* ------------------------------------------------------------------------ */
/* Neural radiance cache (no reference counterpart)                         */
/* ------------------------------------------------------------------------ */
/* A 64 -> 5 x 64 (ReLU) -> 3 MLP, BF16 weights and activations with FP32
 * accumulation on tensor cores, no biases.  Inputs: a 16-level frequency
 * encoding of the box position (per level sin and cos of 2 pi f_l d_l . p,
 * f_l = 2^(l/2), d_l a fixed spherical Fibonacci direction) and real
 * spherical harmonics of 4 bands (l = 0..3, 16 coefficients: "degree 4"
 * counted in bands) of the view and sun directions.  Output: radiance
 * leaving a scattering vertex toward the
 * viewer.  Weight layout: 5 hidden matrices [in][out] 64x64 row-major, then
 * the output matrix [64][16] (columns 3..15 zero), 21504 floats. */
typedef struct vcr_nrc_params {
  uint32_t train_samples;  /* training records per step (65,536 in the NRC configuration) */
  float learning_rate;     /* Adam step size (1e-3) */
  uint32_t query_capacity; /* cache queries per pass (>= paths of a pass) */
  uint32_t seed;           /* weight initialisation */
  float ema_decay;         /* 0: queries use the training weights; in (0,1):
                              they use a moving average of them with this
                              decay (ramped in as min(d, (1+k)/(10+k))) */
  float tail_survival;     /* 0: training paths run to escape / max_events;
                              in (0,1): after their last recorded vertex they
                              continue each event with this probability and
                              weight 1/p (Russian roulette: unbiased targets,
                              a shorter latency tail) */
  uint32_t query_kernel;   /* VCR_NRC_QUERY_*: which tensor-core kernel
                              serves the cache's queries */
  uint32_t position_drop;  /* 0..16: the finest frequency levels of the
                              position encoding whose inputs are held at 0
                              (0: all 16 levels, 16: no position input; for
                              measuring what the encoding contributes) */
  uint32_t encoding;       /* VCR_NRC_ENCODING_*: how the 32 position inputs
                              are formed */
} vcr_nrc_params;

/* Position encodings of the cache (the 16 levels' 2 inputs each):
 * FREQUENCY (default): sin and cos of 2 pi 2^(l/2) d_l . p along a fixed
 * direction d_l per level.  GRID: a multiresolution grid, level l with
 * floor(16 * 64^(l/15)) cells per box axis (16 .. 1024) and a table of
 * 2^17 entries of 2 trainable features (dense for levels 0..4, spatially
 * hashed above), trilinearly interpolated; the 4,194,304 table values are
 * parameters after the network's weights (vcr_nrc_get_weights and the
 * gradient take either the weight count or the full count, which
 * vcr_nrc_info reports) and take Adam steps 10x the network's size. */
#define VCR_NRC_ENCODING_FREQUENCY 0u
#define VCR_NRC_ENCODING_GRID 1u

#define VCR_NRC_QUERY_DEFAULT 0u  /* the library's choice (the faster measured) */
#define VCR_NRC_QUERY_MMA 1u      /* warp-level mma.sync, 16-record tiles per warp */
#define VCR_NRC_QUERY_TCGEN05 2u  /* tcgen05.mma, 128-record tiles, TMEM accumulators */

typedef struct vcr_nrc_info_t {
  uint32_t steps;         /* Adam steps taken */
  float last_loss;        /* relative L2 loss of the last step */
  uint32_t train_records; /* training records of the last step */
  uint32_t queries;       /* cache queries of the last pass */
  uint32_t weights;       /* parameter count (network weights, then the grid encoding's tables) */
} vcr_nrc_info_t;

VCR_API vcr_status vcr_nrc_setup(vcr_ctx* ctx, const vcr_nrc_params* p);
VCR_API vcr_status vcr_nrc_free(vcr_ctx* ctx);
/* One online training step: training paths from the current camera
 * (unbiased, full length) record the radiance leaving their first
 * scattering vertices; the fused kernel computes the relative L2 loss
 * gradient; Adam updates the weights.  With vcr_params.nrc_events = k > 0,
 * vcr_pt_pass (DDA tracker) ends paths at their k-th scattering event and
 * adds throughput x cache prediction there.  pass.spp = S > 1 traces S
 * training sets (about S x train_samples records) in the one launch, for
 * vcr_nrc_train_more to walk: a training-only launch lasts as long as its
 * longest path, so S sets cost far less than S steps (S <= 64,
 * S x train_samples <= 2^24; the record buffer grows on first use). */
VCR_API vcr_status vcr_nrc_train_step(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
/* One frame of the cached tracker, the same as vcr_pt_pass followed by
 * vcr_nrc_train_step with the same pass: one wavefront launch runs the
 * frame's training paths (which never read the weights) first and the
 * pass's camera paths after them, so the long training paths overlap the
 * short camera paths; the camera paths end in the cache, answered with the
 * weights before this frame's update; then the gradient and Adam step.
 * Needs the DDA tracker and params.nrc_events > 0. */
VCR_API vcr_status vcr_nrc_frame(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
/* `steps` further gradient + Adam steps on the records of the last training
 * step (all its sets) or frame (a cheap warm-up: the records are reused,
 * not re-traced).  A step of several sets takes its own Adam step on their
 * first train_samples records.
 * max_records > 0 makes each step use a batch of that many records, the
 * steps (and the next calls) walking through the records batch by batch
 * until new records are traced; 0 uses them all. */
VCR_API vcr_status vcr_nrc_train_more(vcr_ctx* ctx, uint32_t steps, uint32_t max_records, void* stream);
/* Adam step size for the following steps (> 0); the moments are kept. */
VCR_API vcr_status vcr_nrc_set_learning_rate(vcr_ctx* ctx, float learning_rate);
VCR_API vcr_status vcr_nrc_info(vcr_ctx* ctx, vcr_nrc_info_t* out);
VCR_API vcr_status vcr_nrc_get_weights(vcr_ctx* ctx, float* host_out, size_t count);
VCR_API vcr_status vcr_nrc_set_weights(vcr_ctx* ctx, const float* host, size_t count);
/* Cache predictions for n device records (64-byte records: position,
 * direction toward the viewer, sun direction as float3 each, then 3 floats
 * and 4 words unused here); 3 floats per record. */
VCR_API vcr_status vcr_nrc_forward(vcr_ctx* ctx, const void* d_records, uint32_t n, float* d_out, void* stream);
/* `steps` Adam steps on n caller-provided device records (the 3 floats
 * after the directions are the targets): offline fitting and warm starts. */
VCR_API vcr_status vcr_nrc_fit(vcr_ctx* ctx, const void* d_records, uint32_t n, uint32_t steps, void* stream);
/* Loss gradient over n device records (the 3 floats after the directions
 * are the targets) without a weight update; synchronous. */
VCR_API vcr_status vcr_nrc_gradient(vcr_ctx* ctx, const void* d_records, uint32_t n, float* host_grad,
                                    size_t count, float* out_loss);

/* ------------------------------------------------------------------------ */
/* Volumetric progressive photon mapping (RenderTechniquePPM)               */
/* ------------------------------------------------------------------------ */
typedef struct vcr_ppm_params {
  uint32_t photons;  /* photons emitted per pass (200 x 64 in RenderTechniquePPM.cpp:253) */
  uint32_t capacity; /* photons stored per pass (every real collision); extra are dropped */
  float radius;      /* initial gather radius R0, world units (initialRadius) */
  float alpha;       /* radius reduction (m_alpha, RenderTechniquePPM.h:66) */
  uint32_t estimator;  /* VCR_PPM_GATHER or VCR_PPM_MARCH */
  float march_step;    /* VCR_PPM_MARCH: step of the camera-ray march, world units
                          (stepSize, UniformBuffers.h:221) */
  float ambient_step;  /* VCR_PPM_MARCH: step of the ambient march toward the sky
                          (sampleDist, PPM_PE.comp:513) */
} vcr_ppm_params;

/* The radiance estimate of a pass.
 * VCR_PPM_GATHER: stochastic progressive photon mapping -- one delta-tracked
 *   measurement point per pixel, per-pixel radius and flux statistics in
 *   FP64 (N' = N + alpha M, R' = R ((N + alpha M)/(N + M))^(1/3)).
 * VCR_PPM_MARCH: the reference's estimate (PPM_PE.comp:443-546): a march
 *   back to front along the camera ray with march_step (start jittered);
 *   at each step the shadow volume's transmittance times the phase
 *   function toward the sun, an ambient term (the sky along a phase-sampled
 *   direction, attenuated by a march of ambient_step to the box), and the
 *   photon map within one global radius per pass (RenderTechniquePPM.cpp
 *   :302-312: r_1 = R0, r_k = r_(k-1) ((k - 1 + alpha) / k)^0.33333);
 *   L = L exp(-sigma_t step) + sigma_s (direct + indirect) step.  Needs
 *   vcr_shadow_volume_build; the per-pixel statistics are not used; each
 *   pass's estimate is added to the sums (the reference's running mean). */
#define VCR_PPM_GATHER 0u
#define VCR_PPM_MARCH 1u

typedef struct vcr_ppm_info_t {
  uint32_t photons_stored; /* photons in the last pass's tree */
  uint32_t dropped;        /* photons beyond the capacity in the last pass */
} vcr_ppm_info_t;

typedef enum vcr_ppm_buffer {
  VCR_PPM_STATS = 0, /* float64 x8 per pixel: N, R, tau rgb, background-sum rgb */
  VCR_PPM_POS = 1,   /* float4 per stored photon (append order) */
  VCR_PPM_POWER = 2, /* float4 per stored photon: arriving power rgb */
  VCR_PPM_DIR = 3,   /* float4 per stored photon: travel direction */
  VCR_PPM_UID = 4,   /* uint32 per stored photon: photon * 64 + event */
  VCR_PPM_ORDER = 5, /* uint32 per tree leaf: stored photon of the leaf */
  VCR_PPM_LEFT = 6,  /* uint32 per internal node (bit 31 = leaf) */
  VCR_PPM_RIGHT = 7
} vcr_ppm_buffer;

/* Allocate photon buffers and per-pixel statistics for the current frame;
 * resets the sums (RenderTechniquePPM::AllocateResources, :115-156). */
VCR_API vcr_status vcr_ppm_setup(vcr_ctx* ctx, const vcr_ppm_params* p);
VCR_API vcr_status vcr_ppm_free(vcr_ctx* ctx);
/* One pass (RecordDrawCommands, RenderTechniquePPM.cpp:229-300): photon
 * emission with a deposit at every real collision (PPM_PT.comp), photon
 * tree over the Morton-sorted photons (the KDTree the reference stubs,
 * KDTree.cpp:6-79), per-pixel measurement point + radius query
 * (samplePhotonMap, PPM_PE.comp:304-375) and the FP64 N/R/flux update
 * (in place of the global UpdateRadius, :302-312).  The sums then hold the
 * current estimate times the pass count. */
VCR_API vcr_status vcr_ppm_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
VCR_API vcr_status vcr_ppm_info(vcr_ctx* ctx, vcr_ppm_info_t* out);
/* The last pass's gather kernel: leaf photons it tested against the
 * pixels' radii and its device time (two events around the launch).
 * Waits for the gather to finish.  No reference counterpart (measurement). */
VCR_API vcr_status vcr_ppm_gather_stats(vcr_ctx* ctx, uint64_t* photons_tested, float* ms);
VCR_API vcr_status vcr_ppm_read(vcr_ctx* ctx, vcr_ppm_buffer which, void* host_out, size_t bytes);

/* ------------------------------------------------------------------------ */
/* Progressive photon beams (RenderTechniquePPB, RenderTechniquePPB.cpp)    */
/* ------------------------------------------------------------------------ */
typedef struct vcr_ppb_params {
  uint32_t photons;  /* photons emitted per pass (m_beamsPerPass, RenderTechniquePPB.h:117-120) */
  uint32_t capacity; /* beam segments per pass (BVH leaves; m_maxBeamCount :116); extra are dropped */
  float radius;      /* initial beam radius r0, world units (initialRadius, main.cpp:814) */
  float alpha;       /* radius reduction (m_alpha, RenderTechniquePPB.h:114) */
} vcr_ppb_params;

typedef struct vcr_ppb_info_t {
  uint32_t segments;   /* beam segments (BVH leaves) of the last pass */
  uint32_t dropped;    /* segments beyond the capacity in the last pass */
  float radius;        /* radius used by the last pass */
  uint32_t beam_slots; /* beams a photon can deposit (events + 1) */
} vcr_ppb_info_t;

typedef enum vcr_ppb_buffer {
  VCR_PPB_SLOTS = 0,    /* float x28 per (photon, beam): start, dir, length, power, 16 distances */
  VCR_PPB_NBEAMS = 1,   /* uint32 per photon */
  VCR_PPB_SEG_A = 2,    /* float4 per segment: start, radius */
  VCR_PPB_SEG_B = 3,    /* float4 per segment: end, offset along its beam */
  VCR_PPB_SEG_BEAM = 4, /* uint32 per segment: beam slot */
  VCR_PPB_CODES = 5,    /* uint32 per segment: 30-bit Morton code (unsorted) */
  VCR_PPB_ORDER = 6,    /* uint32 per leaf: segment of each sorted leaf */
  VCR_PPB_LEFT = 7,     /* uint32 per internal node (bit 31 = leaf) */
  VCR_PPB_RIGHT = 8,
  VCR_PPB_NODE_LO = 9,  /* float4 per internal node */
  VCR_PPB_NODE_HI = 10,
  VCR_PPB_LEAF_LO = 11, /* float4 per leaf */
  VCR_PPB_LEAF_HI = 12
} vcr_ppb_buffer;

/* Allocate the beam buffers (RenderTechniquePPB::AllocateResources,
 * RenderTechniquePPB.cpp:282-355); beams hold max_events + 1 slots per
 * photon, so call after vcr_set_params. */
VCR_API vcr_status vcr_ppb_setup(vcr_ctx* ctx, const vcr_ppb_params* p);
/* FreeResources (RenderTechniquePPB.cpp:282-355). */
VCR_API vcr_status vcr_ppb_free(vcr_ctx* ctx);
/* One progressive pass (RecordDrawCommands, RenderTechniquePPB.cpp:436-519):
 * photon emission with beam deposit (PPB_PT.comp), segmenting + 30-bit
 * Morton keys, radix sort, LBVH build (PPB_GenerateHierarchy.comp), AABB
 * refit (PPB_CalculateAABB.comp), per-pixel beam gather (PPB_PE.comp); the
 * radius of pass k is r0 prod_{i=1..k} (i + alpha)/(i + 1) (UpdateRadius,
 * :530-546).  One estimate per pixel is added to the FP64 sums. */
VCR_API vcr_status vcr_ppb_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
VCR_API vcr_status vcr_ppb_info(vcr_ctx* ctx, vcr_ppb_info_t* out);
/* The last pass's gather kernel: (pixel, beam segment) pairs it evaluated
 * (segments whose box the pixel's ray hit) and its device time.  Waits for
 * the gather to finish.  No reference counterpart (measurement). */
VCR_API vcr_status vcr_ppb_gather_stats(vcr_ctx* ctx, uint64_t* segments_evaluated, float* ms);
/* Synchronous copy of one of the last pass's beam buffers. */
VCR_API vcr_status vcr_ppb_read(vcr_ctx* ctx, vcr_ppb_buffer which, void* host_out, size_t bytes);
/* LBVH over n Morton-sorted segments (device buffers): Karras build with
 * index-augmented prefixes for equal keys, then capped-cylinder leaf boxes
 * and the bottom-up refit.  d_order[i] = segment of sorted leaf i;
 * segments are float4 (start, radius) and float4 (end, any).  Internal node
 * children carry bit 31 for leaves.  Replaces PPB_GenerateHierarchy.comp
 * (:122-168) + PPB_CalculateAABB.comp (:100-120). */
VCR_API vcr_status vcr_lbvh_build(vcr_ctx* ctx, const uint32_t* d_sorted_codes, const uint32_t* d_order,
                                  const float* d_seg_a, const float* d_seg_b, uint32_t n, uint32_t* d_left,
                                  uint32_t* d_right, float* d_node_lo, float* d_node_hi, float* d_leaf_lo,
                                  float* d_leaf_hi, void* stream);

/* ------------------------------------------------------------------------ */
/* Photon-beam ordering primitives                                          */
/* ------------------------------------------------------------------------ */
/* Stable LSD radix sort of (uint32 key, uint32 value) pairs over key bits
 * [begin_bit, end_bit) (8-bit digit passes: the stable order the
 * reference's 4-bit passes give, in half the passes); device pointers,
 * n <= 2^30 - 1.
 * d_vals_in == NULL sorts the indices 0..n-1 as values (a permutation).
 * Keys (and values) may be sorted in place.  Scratch comes from the
 * context (about 8 bytes per key).
 * Replaces: PPB_RadixSort_LocalSort.comp (:154-252) + PPB_RadixSort_PrefixSum
 * .comp (:28-37) + PPB_RadixSort_GlobalSort.comp (:54-106), dispatched by
 * RenderTechniquePPB::RecordDrawCommands (RenderTechniquePPB.cpp:465-491). */
VCR_API vcr_status vcr_radix_sort_pairs(vcr_ctx* ctx, const uint32_t* d_keys_in, const uint32_t* d_vals_in,
                                        uint32_t* d_keys_out, uint32_t* d_vals_out, uint32_t n,
                                        uint32_t begin_bit, uint32_t end_bit, void* stream);
/* The same sort for callers that cannot allocate device memory (a host
 * application that owns all device memory through its own pool, a render
 * loop that must not allocate after start-up, a plug-in handed buffers but
 * no allocator).  No counterpart in the reference.  It takes no context and
 * allocates nothing: its working memory is one fixed device array (about
 * 9.4 MB) inside this library, held by every GPU that loads it until the
 * process exits.  At most VCR_SORT_NOALLOC_MAX_KEYS pairs per call (larger
 * n returns VCR_ERR_CAPACITY).  Calls share that array: calls that overlap
 * on the GPU race, so serialise them.  The first call on each device looks
 * up the array's address with that device current; make it before any
 * stream capture.  Argument errors are reported through
 * vcr_last_error(NULL); a device-side wait that ran out is reported by
 * vcr_sort_noalloc_status. */
#define VCR_SORT_NOALLOC_MAX_KEYS (1u << 20)
VCR_API vcr_status vcr_radix_sort_pairs_noalloc(const uint32_t* d_keys_in, const uint32_t* d_vals_in,
                                                uint32_t* d_keys_out, uint32_t* d_vals_out, uint32_t n,
                                                uint32_t begin_bit, uint32_t end_bit, void* stream);
/* Waits for `stream`, then reads and clears the device error word of the
 * allocation-free sort on the current device: VCR_ERR_TIMEOUT if a
 * look-back wait of a sort queued before ran out (its output order is then
 * unspecified), else VCR_OK.  Allocates nothing. */
VCR_API vcr_status vcr_sort_noalloc_status(void* stream);
/* Morton codes of n points (device float3): bits == 30 quantises each axis
 * to 1024 cells of [bounds_min, bounds_max] and interleaves x<<2|y<<1|z;
 * bits == 24 is the reference's getMortonCode (PPB_PT.comp:317-333:
 * (p - bounds_min)/256 clamped to [0,255] per axis). */
VCR_API vcr_status vcr_morton_codes(vcr_ctx* ctx, const float* d_points, uint32_t n, const float bounds_min[3],
                                    const float bounds_max[3], uint32_t bits, uint32_t* d_codes, void* stream);

/* ------------------------------------------------------------------------ */
/* Batched multi-view tracking                                              */
/* ------------------------------------------------------------------------ */
/* Many views, each a camera with its own frame size and sun direction, in
 * one persistent DDA-wavefront launch over one work range.  The reference
 * dispatches one camera per RecordDrawCommands (RenderTechniquePT.cpp:
 * 129-168); a batch pass is that dispatch for every view at once.  View v
 * draws its streams with seed + v * 0x9E3779B9, keyed by its own pixel
 * index and the pass like vcr_pt_pass, so each view equals a single-view
 * pass with that seed.  The scene (grid, cloud, params except the sun) is
 * the context's; params must select the DDA tracker, PCG streams, ratio
 * NEE and no cache. */
typedef struct vcr_view_desc {
  vcr_camera camera;
  uint32_t width, height;
  float sun_dir[3];   /* direction the sunlight travels (unit) */
  uint32_t reserved;
} vcr_view_desc;

typedef struct vcr_batch_info_t {
  uint32_t views;
  uint32_t passes;
  uint64_t pixels;   /* all views */
  uint64_t samples;  /* camera samples per pixel summed over passes */
} vcr_batch_info_t;

/* 1..256 views, < 2^31 pixels in all; allocates the FP64 sums. */
VCR_API vcr_status vcr_batch_setup(vcr_ctx* ctx, const vcr_view_desc* views, uint32_t count);
VCR_API vcr_status vcr_batch_free(vcr_ctx* ctx);
/* One pass over every view (pass->spp samples per pixel; crop and flags
 * must be zero). */
VCR_API vcr_status vcr_batch_pass(vcr_ctx* ctx, const vcr_pass_desc* pass, void* stream);
/* Record one batch pass as a CUDA graph (synchronous).  Each replay renders
 * the next pass index, starting at pass->pass_index; a later pass with a
 * different spp drops the graph. */
VCR_API vcr_status vcr_batch_graph_record(vcr_ctx* ctx, const vcr_pass_desc* pass);
VCR_API vcr_status vcr_batch_graph_replay(vcr_ctx* ctx, uint32_t count, void* stream);
/* Times a batch pass per candidate tuning (majorant level x DDA cells per
 * wavefront step x CTA size), keeps the fastest, clears the sums. */
VCR_API vcr_status vcr_batch_autotune(vcr_ctx* ctx, const vcr_pass_desc* pass, vcr_tuning* out, void* stream);
/* FP64 RGB sums of one view (width * height * 3 doubles; host or device
 * memory). */
VCR_API vcr_status vcr_batch_read(vcr_ctx* ctx, uint32_t view, double* out, size_t bytes);
VCR_API vcr_status vcr_batch_info(vcr_ctx* ctx, vcr_batch_info_t* out);
VCR_API vcr_status vcr_batch_reset(vcr_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* Checkpoint / resume of the progressive state                             */
/* ------------------------------------------------------------------------ */
/* Saves the frame's FP64 sums and pass/sample counts, the PPM per-pixel
 * statistics, the radiance cache's weights and Adam state, and a batch's
 * sums, whichever exist (the reference keeps frameCount, the accumulated
 * image and pmRadius only in memory: main.cpp:262, PathTracer.comp:420-424,
 * RenderTechniquePPM.cpp:302-312).  Written to path + ".partial" and renamed
 * when complete.  Synchronous. */
VCR_API vcr_status vcr_checkpoint_save(vcr_ctx* ctx, const char* path);
/* Restores a checkpoint into a context set up the same way (frame size,
 * techniques and their sizes); the grid, cloud, camera and params are the
 * caller's to bind.  The file carries a hash of the scene it was rendered
 * from (grid description, precision and per-brick majorants; cloud,
 * camera and params; batch views and photon-map parameters when set up):
 * a context bound to another scene gets VCR_ERR_STATE.  Every section is
 * checked before anything changes; a truncated or corrupt file is
 * VCR_ERR_IO. */
VCR_API vcr_status vcr_checkpoint_load(vcr_ctx* ctx, const char* path);

/* ------------------------------------------------------------------------ */
/* Read back                                                                */
/* ------------------------------------------------------------------------ */
/* Synchronous copy of a context buffer (bytes must match). host_out may be
 * host, pinned or device memory of the context's device. */
VCR_API vcr_status vcr_readback(vcr_ctx* ctx, vcr_buffer_id id, void* host_out, size_t bytes);
/* Stream-ordered read back of VCR_BUF_IMAGE_MEAN (FP32 RGB, W*H*12 bytes)
 * or VCR_BUF_IMAGE_SUM (FP64, W*H*24 bytes): the image as it stands after
 * the work queued on `stream` is staged on `stream` (into one of two
 * device slots) and copied to host_out on the context's own copy stream,
 * so that the next pass queued on `stream` runs while the copy does.
 * host_out should be pinned (page-locked) memory and must stay untouched
 * until vcr_readback_wait returns; two calls in flight need two host
 * buffers.  Replaces the per-frame transfer of the result image
 * (RenderTechniquePT.cpp:143-167 blits it to the swapchain instead). */
VCR_API vcr_status vcr_readback_async(vcr_ctx* ctx, vcr_buffer_id id, void* host_out, size_t bytes, void* stream);
/* Blocks until every copy queued by vcr_readback_async has landed. */
VCR_API vcr_status vcr_readback_wait(vcr_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* Display image                                                            */
/* ------------------------------------------------------------------------ */
/* Replaces the blit of the result image into the swapchain
 * (RenderTechniquePT.cpp:143-167; the swapchain is B8G8R8A8_SRGB,
 * VulkanSwapchain.cpp:72, so the blit clamps to [0, 1] and sRGB-encodes):
 * every pixel's accumulated mean times `exposure` (1 = the reference),
 * clamped to [0, 1], sRGB-encoded (IEC 61966-2-1) and rounded to 8 bits,
 * alpha 255, as R G B A bytes or, with VCR_ORDER_BGRA, as the swapchain's
 * B G R A. */
typedef enum vcr_pixel_order { VCR_ORDER_RGBA = 0, VCR_ORDER_BGRA = 1 } vcr_pixel_order;
typedef struct vcr_display_desc {
  float exposure;
  uint32_t order; /* vcr_pixel_order */
  uint32_t reserved[2];
} vcr_display_desc;
/* out: W*H*4 bytes.  Device memory of the context's device: written in
 * stream order.  Host memory: written when the call returns. */
VCR_API vcr_status vcr_display(vcr_ctx* ctx, const vcr_display_desc* desc, void* out, size_t bytes, void* stream);
/* Number of passes accumulated into the sums so far. */
VCR_API vcr_status vcr_pass_count(vcr_ctx* ctx, uint32_t* out);
/* Relative RMSE of the running mean image I against a reference mean image
 * R (device, FP64 RGB, W*H*3):
 *     sqrt( mean_p sum_c (I - R)^2 / (R^2 + 1e-2) ),
 * written as one double to d_out (device). Stream-ordered and asynchronous,
 * so an error curve can be recorded after every pass without a host sync.
 * No reference counterpart (the reference only displays the image). */
VCR_API vcr_status vcr_image_rel_rmse(vcr_ctx* ctx, const double* d_ref, double* d_out, void* stream);

/* ------------------------------------------------------------------------ */
/* Image files (host memory, synchronous, no GPU needed)                    */
/* ------------------------------------------------------------------------ */
/* Where the reference shows the result in its window, a headless renderer
 * writes files.  vcr_write_exr: the HDR image (W*H*3 floats, RGB, rows top
 * to bottom: what vcr_readback(VCR_BUF_IMAGE_MEAN) returns) as an OpenEXR
 * 2.0 file — single part, scan lines, no compression, channels B, G, R of
 * pixel type VCR_EXR_HALF (rounded to nearest, ties to even; past 65504 it
 * is infinity) or VCR_EXR_FLOAT.  vcr_write_png: W*H*4 bytes of 8-bit RGBA
 * (vcr_display's VCR_ORDER_RGBA output) as a PNG file with stored
 * (uncompressed) deflate blocks, so that no compression library is needed. */
typedef enum vcr_exr_type { VCR_EXR_HALF = 1, VCR_EXR_FLOAT = 2 } vcr_exr_type;
VCR_API vcr_status vcr_write_exr(const char* path, uint32_t width, uint32_t height, const float* rgb,
                                 uint32_t type);
VCR_API vcr_status vcr_write_png(const char* path, uint32_t width, uint32_t height, const uint8_t* rgba);

#ifdef __cplusplus
}
#endif

#endif /* VCR_ABI_H */

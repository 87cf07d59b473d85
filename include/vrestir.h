/* vrestir.h -- C ABI of the GB300-native Volumetric ReSTIR frame loop (libvrestir.so).
 *
 * This library replaces the per-frame path of the `VolumetricReSTIR` render pass of
 * DQLin/VolumetricReSTIRRelease.  Each entry point names the reference interface it stands
 * in for (paths relative to the reference repository):
 *
 *   plugin discovery / create  Source/RenderPasses/VolumetricReSTIR/VolumetricReSTIR.cpp:61-70
 *                              (getPasses -> VolumetricReSTIR::create(RenderContext*, Dictionary))
 *   options                    VolumetricReSTIR.h:130-207 (VolumetricReSTIRParams),
 *                              VolumetricReSTIR.cpp:1280-1347 (setDictionary / option changes)
 *   scene binding              VolumetricReSTIR.cpp:1218-1256 (setScene), Falcor Scene.cpp:2754
 *                              (Scene::addGVDBVolume), EnvMapSampler.cpp:39-100 (importance map)
 *   per-frame call             Source/Falcor/RenderGraph/RenderPass.h:114 (execute), implemented by
 *                              VolumetricReSTIR.cpp:303-906; output channel `accumulated_color`
 *   reservoir layout           HostDeviceSharedDefinitions.h:16-71 (Reservoir, ExtraBounceReservoir,
 *                              ReservoirFeatures)
 *
 * Conventions: every function returns an int status (VR_OK = 0) unless stated otherwise;
 * exceptions never cross this boundary.  A context owns all of its device buffers; output
 * pointers are owned by the caller.  A context is not thread-safe; separate contexts may be
 * used from separate threads.  All GPU work of a call is issued on the caller's stream
 * (a cudaStream_t passed as void*; NULL = legacy default stream).
 */
#ifndef VRESTIR_H
#define VRESTIR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (reference: exceptions / logError, VolumetricReSTIR.cpp:196) ---- */
#define VR_OK 0
#define VR_ERR_INVALID_ARG 1
#define VR_ERR_OOM 2
#define VR_ERR_CUDA 3
#define VR_ERR_LOOP_LIMIT 4     /* a bounded device loop hit its limit (status word set) */
#define VR_ERR_UNSUPPORTED 5    /* option value outside the supported surface */
#define VR_ERR_STATE 6          /* call order: e.g. render before a volume is bound */

/* ---- enums, values as in HostDeviceSharedConstants.slang:5-16, 29-31 ---- */
#define VR_MIS_NONE 0
#define VR_MIS_TALBOT 1
#define VR_SAMPLER_HAMMERSLEY 0
#define VR_SAMPLER_R2 1
#define VR_TRACK_RATIO 0
#define VR_TRACK_ANALYTIC 1
#define VR_TRACK_RAY_MARCHING 2
#define VR_TRACK_RESIDUAL_RATIO 3
#define VR_TRACK_ANALOG_RESIDUAL_RATIO 4
#define VR_REPROJ_LINEAR 0
#define VR_REPROJ_NONE 1
#define VR_REPROJ_NO_BACKGROUND 2

#define VR_NUM_MAX_MIPS 8           /* kNumMaxMips; slots 0-7 normal, 8-15 conservative */
#define VR_NUM_SLOTS 16
#define VR_MAX_BOUNCES 4            /* max path length supported by this build */
#define VR_BRICK 8                  /* brick edge in voxels */
#define VR_BRICK_APRON 10           /* stored brick edge: 8 + 2 x apron of 1 */

/* Options: same names, meanings and defaults as VolumetricReSTIRParams
 * (VolumetricReSTIR.h:130-207).  Members absent here (surface scenes, mesh lights) are outside
 * this path; animation is set with vr_set_animation.  vr_options_default() fills the defaults. */
typedef struct vr_options {
    int32_t mMaxBounces;                        /* 1 */
    int32_t mEnableTemporalReuse;               /* 1 */
    int32_t mEnableSpatialReuse;                /* 1 */
    int32_t mUseReference;                      /* 0: volume path tracer instead of ReSTIR */
    int32_t mUseEnvironmentLights;              /* 1 */
    int32_t mUseAnalyticLights;                 /* 0 */
    int32_t mBaselineSamplePerPixel;            /* 1 */
    int32_t mVisualizeTotalTransmittance;       /* 0 */
    int32_t mInitialBaseMipLevel;               /* 1 */
    int32_t mInitialM;                          /* 4 */
    int32_t mInitialLightSamples;               /* 1 */
    int32_t mInitialLightingMipLevel;           /* 2 */
    int32_t mInitialVisibilityUseLinearSampler; /* 0 */
    int32_t mInitialLightingUseLinearSampler;   /* 1 */
    uint32_t mInitialLightingTrackingMethod;    /* VR_TRACK_RAY_MARCHING */
    float mInitialVisibilityTStepScale;         /* 1 */
    float mInitialLightingTStepScale;           /* 2 */
    int32_t mInitialUseRussianRoulette;         /* 1 */
    int32_t mInitialUseCoarserGridForIndirectBounce; /* 1 */
    float mTemporalReuseMThreshold;             /* 4 */
    uint32_t mTemporalReprojectionMode;         /* VR_REPROJ_LINEAR */
    uint32_t mTemporalMISMethod;                /* VR_MIS_TALBOT */
    int32_t mTemporalReprojectionMipLevel;      /* 1 */
    int32_t mSpatialReuseRounds;                /* 1 */
    int32_t mSpatialVisibilityMipLevel;         /* 1 */
    int32_t mSpatialLightingMipLevel;           /* 1 */
    int32_t mSpatialVisibilityUseLinearSampler; /* 1 */
    int32_t mSpatialLightingUseLinearSampler;   /* 1 */
    float mSpatialVisibilityTStepScale;         /* 1 */
    float mSpatialLightingTStepScale;           /* 1 */
    uint32_t mSpatialVisibilityTrackingMethod;  /* VR_TRACK_RAY_MARCHING */
    uint32_t mSpatialLightingTrackingMethod;    /* VR_TRACK_RAY_MARCHING */
    uint32_t mRandomSamplerType;                /* VR_SAMPLER_R2 */
    float mSampleRadius;                        /* 10 */
    int32_t mSpatialSampleCount;                /* 4 (includes the centre pixel) */
    uint32_t mSpatialMISMethod;                 /* VR_MIS_TALBOT */
    int32_t mFinalLightSamples;                 /* 1 */
    int32_t mFinalVisibilitySamples;            /* 1 */
    uint32_t mFinalVisibilityTrackingMethod;    /* VR_TRACK_ANALYTIC */
    uint32_t mFinalLightTrackingMethod;         /* VR_TRACK_ANALYTIC */
    float mFinalTStepScale;                     /* 0.2 */
    /* Learned target function for the initial candidates (no counterpart in the reference):
     * a transmittance MLP replaces the marched light visibility inside the initial RIS target
     * (ComputeInitialSample.slang's SampleDirectLighting shadow ray).  The marched estimators
     * keep evaluating every later p_hat (TraceRays.cs.slang:176-183, temporal, spatial) and the
     * final shading, so the estimator stays unbiased for any network.  Needs temporal or
     * spatial reuse. */
    int32_t mUseLearnedPHat;                    /* 0 */
    int32_t mLearnedTrainSamples;               /* 1048576 new training samples per frame (0: frozen) */
    int32_t mLearnedBatch;                      /* 16384 samples per Adam step */
    float mLearnedLearningRate;                 /* 1e-3 */
    float mLearnedTFloor;                       /* 0.02: lower clamp of the predicted transmittance */
    uint32_t mLearnedSeed;                      /* 1: weight initialisation and training streams */
    uint32_t mLearnedTargetMethod;              /* VR_TRACK_RAY_MARCHING: estimator of the training targets (mip 0) */
    int32_t mLearnedLoss;                       /* 0: squared error of T; 1: squared error of log T (targets floored) */
    /* animated volumes (VolumetricReSTIR.h:152): evaluate the temporal tap's MIS weight on the
     * previous animation frame's grids (VolumeDesc.usePrevGridForReproj) */
    int32_t mUsePrevVolumeForReproj;            /* 1 */
    /* vertex reuse (VolumetricReSTIR.h:136-137, the VERTEX_REUSE define): from indirect vertex
     * mVertexReuseStartBounce on, a path's suffix is kept as vertex positions, so spatial reuse
     * reconnects the shifted prefix to the same suffix vertex and reuses the suffix's share of
     * p_hat (p_partial) instead of re-marching it.  Needs mMaxBounces > 1; not with the learned
     * target, batches or the allocation-free frame. */
    int32_t mVertexReuse;                       /* 0 */
    int32_t mVertexReuseStartBounce;            /* 1 */
} vr_options;

/* Participating medium (Scene.cpp:3246-3262 VolumeDesc + addGVDBVolume arguments). */
typedef struct vr_medium {
    float sigma_a[3];
    float sigma_s[3];             /* sigma_t = sigma_a.x + sigma_s.x (grey) */
    float g;                      /* Henyey-Greenstein anisotropy */
    float density_scale;          /* densityScaleFactorByScaling = DensityScale / worldScaling */
} vr_medium;

/* Procedural sparse volume (density in [0,1], fBm Perlin noise): the synthetic stand-in for the
 * reference's .vbx assets.  kind: 0 = fBm x smooth sphere mask (dense), 1 = thresholded fBm
 * (sparse).  The volume occupies the world box [world_min, world_min + res*voxel_size). */
typedef struct vr_procedural_desc {
    int32_t kind;
    int32_t res;                  /* voxels per axis at mip 0 (multiple of 8 * 2^(num_mips-1)) */
    int32_t num_mips;             /* 1..VR_NUM_MAX_MIPS; normal + conservative pyramids */
    int32_t octaves;
    uint32_t seed;
    float lacunarity, gain;
    float base_frequency;         /* noise frequency across the unit cube */
    float mask_radius;            /* kind 0: sphere radius in the unit cube */
    float threshold;              /* kind 1: density = clamp((n - thr)/(1 - thr)) */
    float world_min[3];
    float voxel_size;             /* world size of one mip-0 voxel */
    int32_t fp16;                 /* store bricks as FP16 (precision form) */
} vr_procedural_desc;

typedef struct vr_volume vr_volume;   /* opaque host-side sparse brick grid, all mip slots */

/* Raw view of one mip slot (what the GPU reads and what the oracle consumes). */
typedef struct vr_grid_view {
    int32_t valid;
    int32_t res[3];
    float bmin[3], bmax[3];       /* index-space bounds [0, res) */
    float world_to_index[16];     /* row-vector convention: idx = (p, 1) * M */
    float max_value;              /* max voxel value of this slot */
    int32_t num_l1;
    int32_t num_bricks;
    const int32_t* root_child;    /* 32^3: level-2 child list -> level-1 node, -1 = empty */
    const int32_t* l1_vmin;       /* 4 ints per level-1 node (x, y, z, 0) */
    const int32_t* l1_child;      /* 16^3 per level-1 node -> brick id, -1 = empty */
    const int32_t* brick_vmin;    /* 4 ints per brick */
    const float* brick_bounds;    /* 4 floats per brick: min, max, avg(sum/512), 0 */
    const float* brick_f32;       /* 10^3 floats per brick (apron 1), or NULL */
    const uint16_t* brick_f16;    /* 10^3 halves per brick, or NULL */
    const uint64_t* brick_bc4;    /* 90 BC4 blocks per brick, or NULL (vr_volume_compress_bc4) */
    float bc4_scale;              /* density = decoded unorm value * bc4_scale */
} vr_grid_view;

typedef struct vr_volume_info {
    int32_t num_mips;
    int32_t res;
    float voxel_size;             /* world size of a mip-0 voxel: tStep * worldScaling */
    float supervoxel_diag;        /* superVoxelWorldSpaceDiagonalLength (Scene.cpp:3076-3080) */
    int32_t num_bricks[VR_NUM_SLOTS];
    int64_t device_bytes;         /* bytes the grid occupies once bound to a context */
    int32_t fp16;
    float world_min[3];           /* world position of index-space corner (0, 0, 0) */
    int32_t bc4;                  /* coarse and conservative mips stored as BC4 blocks */
} vr_volume_info;

typedef struct vr_point_light {   /* LightHelpers.slang:223-242 (point light, uniform emission) */
    float pos[3];
    float intensity[3];
} vr_point_light;

/* Lat-long environment map (EnvMap.slang:45-50) with a linear (wrap u / clamp v) lookup. */
typedef struct vr_env_map {
    const float* rgb;             /* width * height * 3 floats, row-major, host memory */
    int32_t width, height;
    float scale[3];               /* intensity * tint */
    float rotation[9];            /* local->world, row-vector convention (EnvMapData.transform) */
} vr_env_map;

typedef struct vr_camera {        /* Camera.cpp:183-189 pinhole frame, no jitter */
    float pos[3];
    float target[3];
    float up[3];
    float fov_y;                  /* radians */
    float near_z, far_z;
} vr_camera;

/* AoS reservoir record exactly as HostDeviceSharedDefinitions.h:16-45 lays it out
 * (32 bytes for max path length 1; 36 bytes with extraBounceStartId otherwise; 40 bytes with
 * p_partial as well under vertex reuse). */
typedef struct vr_reservoir_aos {
    float runningSum;
    float M;
    float depth;
    float p_y;
    float lightUV[2];
    int32_t lightID;
    int32_t sampledPixel;
    int32_t extraBounceStartId;   /* present in the exported stream only if mMaxBounces > 1 */
    float p_partial;              /* present only with mVertexReuse and mMaxBounces > 1 */
} vr_reservoir_aos;

typedef struct vr_context vr_context;

/* ---- options ---- */
void vr_options_default(vr_options* o);                        /* VolumetricReSTIR.h:130-207 */

/* ---- volumes (Scene::addGVDBVolume, Scene.cpp:2754-3279; mips and conservative mips as in
 *      gvdb_volume_gvdb.cpp:2700-2862; brick bounds as in Scene.cpp:2983-3012) ---- */
int vr_volume_create_procedural(const vr_procedural_desc* d, vr_volume** out);
int vr_volume_create_dense(const float* density, int32_t res, int32_t num_mips,
                           const float world_min[3], float voxel_size, int32_t fp16,
                           vr_volume** out);
/* GVDB .vbx files (gvdb-voxel-src/GVDB_FILESPEC.txt; VolumeGVDB::LoadVBX,
 * gvdb_volume_gvdb.cpp:532-700; the files Scene::addGVDBVolume reads, Scene.cpp:2754-3058).
 * Load reads grid 0 (float, one component, uncompressed, GVDB topology, atlas layout, 8^3
 * leaves, no rotation, uniform scale; versions 1.0-2.x), walks its tree from the root and builds
 * num_mips normal and conservative mips from the reachable leaves, over the file's effective
 * voxel box (version x.12) or the leaves' box; world = (index + pretranslation) * scale +
 * translation.  flags: VR_VBX_FP16 stores FP16 bricks; VR_VBX_SIGNED keeps signed values, mip 0
 * only (velocity components).  Grids up to 1024^3 voxels.  Save writes mip 0 of a volume as a
 * version 1.12 file in the three-level layout (log2 dims 3, 4, 5) with a one-voxel apron.
 * vr_volume_vbx_error describes the last failure of either on this thread. */
#define VR_VBX_FP16 1
#define VR_VBX_SIGNED 2
int vr_volume_load_vbx(const char* path, int32_t num_mips, int32_t flags, vr_volume** out);
int vr_volume_save_vbx(const vr_volume* v, const char* path);
const char* vr_volume_vbx_error(void);
/* A signed scalar grid, mip 0 only (velocity components for vr_set_animation): bricks wherever
 * a voxel is nonzero, values stored as given.  values: res^3, x fastest. */
int vr_volume_create_dense_signed(const float* values, int32_t res, const float world_min[3], float voxel_size,
                                  int32_t fp16, vr_volume** out);
/* The reference's default texture form (Scene.cpp:3161-3181, ATLAS_COMPRESSION 2): normal mips
 * 1.. and every conservative mip re-encoded as BC4 unorm blocks scaled by the slot's maximum
 * (4x4 texels of each z-slice of a brick's 10^3 apron box, 90 blocks of 8 bytes per brick);
 * normal mip 0 keeps its FP32 or FP16 storage.  Brick bounds are recomputed from the decoded
 * values; on the conservative mips no nonzero voxel decodes to zero.  In place; a second call
 * changes nothing. */
int vr_volume_compress_bc4(vr_volume* v);
void vr_volume_destroy(vr_volume* v);
int vr_volume_get_info(const vr_volume* v, vr_volume_info* info);
int vr_volume_get_slot(const vr_volume* v, int32_t slot, vr_grid_view* view);

/* Fire plume (synthetic stand-in for the reference's emissive .vbx sequences): a density volume
 * (column widening with height, fBm turbulence, density falling off with height) and a
 * temperature volume (mip 0 only) over the same box, t_min..t_max kelvin inside the plume and
 * 0 outside.  d->kind, mask_radius and threshold are ignored. */
int vr_volume_create_fire(const vr_procedural_desc* d, float t_min, float t_max, vr_volume** density,
                          vr_volume** temperature);
/* Blackbody colours of 50 K .. 6400 K in 50 K steps (128 RGB triples, linear sRGB): Planck's law
 * integrated against the CIE 1931 colour-matching functions (multi-lobe Gaussian fit of Wyman,
 * Sloan and Shirley, 2013), normalised to unit luminance at 6400 K.  The project's own table in
 * the role of the reference's LUT/BlackBodyRadiationRGB_50K-6400K.txt (Scene.cpp:2877-2893). */
void vr_blackbody_lut(float rgb[384]);

/* ---- context lifecycle (getPasses/create, VolumetricReSTIR.cpp:61-70) ---- */
vr_context* vr_create(const vr_options* opts, int32_t width, int32_t height, int32_t* err);
void vr_destroy(vr_context* ctx);
const char* vr_last_error(const vr_context* ctx);
/* Any change resets the history like mOptionsChanged (VolumetricReSTIR.cpp:349-359). */
int vr_set_options(vr_context* ctx, const vr_options* opts);
int vr_get_options(const vr_context* ctx, vr_options* opts);
int vr_resize(vr_context* ctx, int32_t width, int32_t height);

/* ---- scene binding (setScene, VolumetricReSTIR.cpp:1218-1256) ---- */
int vr_set_volume(vr_context* ctx, const vr_volume* vol, const vr_medium* medium);
int vr_set_lights(vr_context* ctx, const vr_point_light* lights, int32_t num_lights,
                  const vr_env_map* env);
/* Volume emission (hasEmissionGrid, LeScale, temperatureCutOff, temperatureScale of
 * Scene::addGVDBVolume, Scene.cpp:2754; Emission / ConvertTempToColor, VolumeBase.slang:
 * 196-232): Le(x) = le_scale * LUT((min(6400, (T(x) - cutoff) * scale) - 25) / 6400), T the
 * trilinear temperature at mip 0, the 128-texel table read with linear filtering between texel
 * centres and clamped at its ends.  lut_rgb: 128 RGB triples or NULL for vr_blackbody_lut's.
 * temperature NULL switches emission off.  Resets the history like an option change. */
int vr_set_emission(vr_context* ctx, const vr_volume* temperature, float le_scale, float cutoff,
                    float scale, const float* lut_rgb);

/* Animated volume sequences (Scene::addGVDBVolumeSequence, Scene.cpp:3329-3354; the per-frame
 * advance of Scene::update, Scene.cpp:825-860; the previous-frame grids of the temporal pass,
 * ReSTIRHelper.slang:95-96, 450-452, TemporalReuse.cs.slang:161-166).
 *
 * frames[0..n): the density volumes of the sequence, each with the res, mip count and voxel size
 * of the volume given to vr_set_volume (whose medium they use), placed anywhere in the world.  temperature: NULL, or n
 * entries (an entry may be NULL: that frame does not emit), read like vr_set_emission's grid
 * with the parameters of the last vr_set_emission call (the reference's defaults 0.005, 1, 100
 * and the built-in table if there was none).  velocity: NULL, or 3n scalar volumes, the x, y
 * and z components of frame i at [3i, 3i+2], in world units per frame; the temporal
 * reprojection moves the reprojected point back by velocity * velocity_scale.
 *
 * Every vr_render_frame advances the sequence by one frame, cyclically; the first rendered frame
 * is frame 0 and the previous frame of frame 0 is frame n-1.  The frames stay resident in device
 * memory.  With mUsePrevVolumeForReproj the temporal tap's MIS weight evaluates the current
 * sample on the previous frame's grids.  n = 0 returns to the static volume.  Resets the history
 * like an option change.  Not available in batches. */
int vr_set_animation(vr_context* ctx, const vr_volume* const* frames, int32_t n, const vr_volume* const* temperature,
                     const vr_volume* const* velocity, float velocity_scale);
/* Index of the animation frame rendered last (-1 before the first frame or without animation). */
int32_t vr_animation_frame(const vr_context* ctx);

/* ---- per-frame call (execute, VolumetricReSTIR.cpp:303-906) ----
 * out_rgba_device: width*height float4 (RGBA32F, `accumulated_color`), device memory.
 * out_mvec_device: optional width*height float2 motion vectors (mOutputMotionVec), or NULL. */
int vr_render_frame(vr_context* ctx, const vr_camera* cam, float* out_rgba_device,
                    float* out_mvec_device, void* stream);
/* Same frame, host output buffer: copies the image back (synchronises the stream). */
int vr_render_frame_host(vr_context* ctx, const vr_camera* cam, float* out_rgba_host,
                         void* stream);
/* Pipelined host output: renders into one of two device staging images and copies it to
 * out_rgba_host on the context's copy stream without waiting, so frame n's copy overlaps frame
 * n+1's kernels (use pinned host memory for a real overlap).  At most two frames are in flight:
 * a call first waits for the copy issued two calls earlier.  out_rgba_host may be read after
 * vr_host_frames_wait, or once the second call after its own has returned.  Bounded-loop errors
 * of the device are reported by vr_host_frames_wait. */
int vr_render_frame_host_async(vr_context* ctx, const vr_camera* cam, float* out_rgba_host, void* stream);
/* Post-process hook: the slot where the reference's graph puts its OptixDenoiser (and an
 * AccumulatePass before it) after the pass (Scripts/run_plume_denoiser.py: accumulated_color ->
 * AccumulatePass -> OptixDenoiser.color, mvec -> OptixDenoiser.mvec).  When set, every
 * vr_render_frame* call invokes fn on the calling thread once the frame's last pass is enqueued,
 * with the output image (RGBA32F, device), the motion vectors (RG32F, device) or NULL, the size
 * and the frame's stream.  fn enqueues its work on that stream and may rewrite the image in place;
 * the host copies of vr_render_frame_host* are enqueued after it.  NULL removes the hook.
 * Batched rendering (vr_batch_*) does not call it. */
typedef void (*vr_frame_hook)(void* user, float* rgba_device, float* mvec_device_or_null, int32_t width, int32_t height,
                              void* stream);
int vr_set_frame_hook(vr_context* ctx, vr_frame_hook fn, void* user);
int vr_host_frames_wait(vr_context* ctx);

/* ---- allocation-free frame (no counterpart in the reference) ----
 * Renders one frame without temporal history into out_rgba_device, keeping every per-pixel
 * intermediate in a fixed static device array (about 6.3 MiB, held by each GPU that loads the
 * library until exit) instead of allocating.  For callers that may not allocate GPU memory at
 * render time: hosts that hand out a fixed device-memory budget up front and forbid later
 * allocations, and real-time loops where a cudaMalloc (which can synchronise the device) would
 * stall a frame.  Limits: at most 65536 pixels, mMaxBounces <= 2, mEnableTemporalReuse,
 * mUseReference and mUseLearnedPHat off; other requests fail with VR_ERR_INVALID_ARG.
 * frame_index seeds the per-pixel RNG and the neighbour offsets like the frame counter.  Calls
 * share the array and the scene constants of the entry point's own kernels, which every call
 * rewrites: calls that overlap on the GPU race and must be serialised by the caller.  The first
 * call on each device looks up the array's address; make it before any stream capture.
 * Context buffers, counters and history are left untouched. */
int vr_render_frame_noalloc(vr_context* ctx, const vr_camera* cam, int32_t frame_index,
                            float* out_rgba_device, void* stream);

/* Block size of the per-pixel kernels: 32, 64 or 128 threads (8 x 4, 8 x 8 or 8 x 16 pixels).
 * Results do not depend on it. */
int vr_set_block_size(vr_context* ctx, int32_t threads);

/* ---- batches (no counterpart in the reference) ----
 * Many contexts -- each with its own volume, view, resolution, options, network and buffers --
 * rendered together: every pass is one persistent launch over a single list of pixel tiles of
 * all instances, and the whole launch sequence of a frame is captured once into a CUDA graph
 * and replayed (re-captured when resolutions, buffers or the launch shape change).  Results are
 * bit-identical to rendering each context alone with vr_render_frame.  All instances must share
 * mMaxBounces, mEnableTemporalReuse, mEnableSpatialReuse and mSpatialReuseRounds, with
 * mUseReference off.  The batch keeps pointers to the contexts; destroy it first. */
typedef struct vr_batch vr_batch;
int vr_batch_create(vr_context* const* ctxs, int32_t n, vr_batch** out);
void vr_batch_destroy(vr_batch* batch);
const char* vr_batch_last_error(const vr_batch* batch);
/* One frame of every instance: cams[i] and outs_device[i] (width_i*height_i float4). */
int vr_batch_render(vr_batch* batch, const vr_camera* cams, float* const* outs_device, void* stream);
int vr_batch_set_graph(vr_batch* batch, int32_t enable);            /* default on */
/* Launch shape of the batched kernels: tiles of tile_w x (128 / tile_w) pixels, a persistent
 * grid of blocks_per_sm blocks per SM. */
int vr_batch_set_launch_shape(vr_batch* batch, int32_t tile_w, int32_t blocks_per_sm);
int vr_batch_get_launch_shape(const vr_batch* batch, int32_t* tile_w, int32_t* tile_h, int32_t* blocks_per_sm);
/* Autotuner: renders one real frame of the batch with each candidate launch shape (tiles 8x16,
 * 16x8, 32x4 x 3, 5, 8 blocks per SM; at most max_trials of them when max_trials > 0), times it
 * with CUDA events and keeps the fastest.  trial_ms (optional) receives the frame times. */
int vr_batch_autotune(vr_batch* batch, const vr_camera* cams, float* const* outs_device, void* stream,
                      float* trial_ms, int32_t max_trials);
/* Kernel launches of the last batch frame (in the captured graph when it is on). */
int32_t vr_batch_last_launch_count(const vr_batch* batch);

/* ---- FP64 converged reference (IntegrateByVolumePathTracing,
 *      VolumePathTracingFunctions.slang:3-131, accumulated like AccumulatePass'
 *      accumulateDouble, Accumulate.cs.slang:100).  Renders num_frames frames of
 *      mBaselineSamplePerPixel paths each, adding each frame's RGB into accum_device
 *      (width*height*3 doubles, device memory, caller-owned and caller-zeroed). ---- */
int vr_render_reference(vr_context* ctx, const vr_camera* cam, int32_t first_frame,
                        int32_t num_frames, double* accum_device, void* stream);

/* ---- state export / import (checkpoint of the history; no hidden sync elsewhere) ----
 * which: 0 = current reservoirs (output of the last frame), 1 = temporal history.
 * host_aos receives width*height records of vr_reservoir_bytes(ctx) bytes. */
int32_t vr_reservoir_bytes(const vr_context* ctx);
int vr_export_reservoirs(vr_context* ctx, int32_t which, void* host_aos, size_t bytes);
/* extra-bounce records (float3 wi_dist, HostDeviceSharedDefinitions.h:49-52),
 * width*height*(mMaxBounces-1)*3 floats. */
int vr_export_extra_bounces(vr_context* ctx, int32_t which, float* host, size_t bytes);
/* features (int noReflectiveSurface, float transmittance), width*height records. */
int vr_export_features(vr_context* ctx, void* host, size_t bytes);
/* Full state blob (all history buffers, frame counter, previous camera). */
int64_t vr_state_bytes(const vr_context* ctx);
int vr_export_state(vr_context* ctx, void* host, size_t bytes);
int vr_import_state(vr_context* ctx, const void* host, size_t bytes);
int32_t vr_frame_count(const vr_context* ctx);

/* ---- instrumentation ---- */
/* Per-kernel device time of the last vr_render_frame (milliseconds), CUDA events. */
int vr_last_timings(const vr_context* ctx, float* ms, int32_t max_entries, int32_t* n);
/* Device time per kernel stage summed over the frames rendered since the last reset, from CUDA
 * events recorded on the caller's stream: 0 initial stage (k_initial, or generate + infer +
 * select with the learned target), 1 spatial/final stage, 2 network training, 3 generate,
 * 4 infer, 5 select (up to 8 entries).  Waits for those events; call it outside a timed
 * region. */
int vr_kernel_time_totals(vr_context* ctx, float* ms, int32_t max_entries, int32_t* frames, int32_t reset);
/* Kernel launches issued by the last vr_render_frame. */
int32_t vr_last_launch_count(const vr_context* ctx);
/* Host->device and device->host bytes moved by the last frame call (scene constants and
 * launch parameters in; the image out for vr_render_frame_host). */
int vr_last_transfer_bytes(const vr_context* ctx, int64_t* h2d, int64_t* d2h);

/* ---- learned target: the transmittance network (no counterpart in the reference) ----
 * Parameters: VR_NET_PARAMS FP32 values, per hidden layer l = 0..3 a [64 out][64 in] weight
 * matrix (layer 0: 60 encoded inputs, 4 zero pads) then 64 biases; then 64 output weights and
 * the output bias.  Inference uses BF16 weights and activations with FP32 accumulation.
 * Queries and samples are records of 8 floats: x, y, z, wx, wy, wz, tmax, target (training) or
 * slot (the frame's own query list).  Positions are normalised to the bound volume's box. */
#define VR_NET_PARAMS 16705
int vr_net_get_params(vr_context* ctx, float* host_params);
/* Replaces the weights and resets the Adam moments and step counter. */
int vr_net_set_params(vr_context* ctx, const float* host_params);
/* T(x, w) = clamp(exp(net(x, w)), mLearnedTFloor, 1) for n device query records into
 * out_device (n floats), on the tensor cores. */
int vr_net_infer(vr_context* ctx, const float* queries_device, int32_t n, float* out_device, void* stream);
/* Mean squared error of T against the targets of n device samples and its gradient
 * (VR_NET_PARAMS floats, host), without changing the weights.  Synchronises. */
int vr_net_gradients(vr_context* ctx, const float* samples_device, int32_t n, float* grads_host, float* loss_host);
/* One Adam step (mLearnedLearningRate, beta 0.9 / 0.999, eps 1e-8) on n device samples. */
int vr_net_train_step(vr_context* ctx, const float* samples_device, int32_t n, float* loss_host);
/* Buffers of the last learned-target frame, copied to host memory:
 * which 0: T per vertex slot, mInitialM * mMaxBounces * width * height floats (slot
 *          (c * mMaxBounces + b) * width * height + pixel; defined where a query was made);
 * which 1: the query list, query_count records of 8 floats (in arbitrary order);
 * which 2: the training samples of the frame, mLearnedTrainSamples records of 8 floats
 *          (tmax < 0 marks a sample whose path left the volume);
 * which 3: the loss of each Adam step of the frame (floats).
 * *count receives the number of records (or floats for 0 and 3). */
int vr_export_learned(vr_context* ctx, int32_t which, void* host, size_t bytes, int64_t* count);

/* ---- self tests: elementary functions and the RNG evaluated by a device kernel, so callers
 *      can check device/host bit equality.  op: 0 exp, 1 log, 2 sin, 3 cos, 4 atan2, 5 acos,
 *      6 pow, 7 sqrt.  In/out are host arrays of n floats. ---- */
int vr_selftest_math(int32_t op, const float* a, const float* b, float* out, int32_t n);
/* One 128x64x64 BF16 tensor-core product (tcgen05, FP32 accumulation in TMEM):
 * D[128x64] = A[128x64] * B[64x64]^T, row-major bf16 inputs, host arrays.  variant 0/1 selects
 * the descriptor stride convention under test. */
int vr_selftest_umma(const uint16_t* A, const uint16_t* B, float* D, int32_t variant);
/* For n pixel cases (px, py, sampleNumber) returns the first `draws` values of sampleNext1D. */
int vr_selftest_rng(const uint32_t* cases, int32_t n, int32_t draws, float* out);

/* ---- fault injection on the host (testing) ----
 * The n-th device allocation that any context makes from now on (n = 0: the next one) fails as
 * if the device were out of memory; the calls then return VR_ERR_OOM and leave the context
 * usable.  n < 0 switches the injection off. */
void vr_debug_fail_allocation(int32_t n);

/* ---- post-process passes around the frame loop (no part of the reference's ReSTIR pass) ----
 * Accumulation (AccumulatePass, Accumulate.cs.slang:55-125): running per-pixel sums of RGBA32F
 * frames in double, single or compensated single precision (AccumulatePass.h:66-71);
 * vr_accumulate adds one frame and, if out_rgba is not NULL, writes the running mean
 * (float)(sum / count).  vr_accumulator_reset restarts the sums. */
#define VR_ACCUM_DOUBLE 0
#define VR_ACCUM_SINGLE 1
#define VR_ACCUM_SINGLE_COMPENSATED 2
typedef struct vr_accumulator vr_accumulator;
int vr_accumulator_create(int32_t width, int32_t height, int32_t precision, vr_accumulator** out);
void vr_accumulator_destroy(vr_accumulator* acc);
void vr_accumulator_reset(vr_accumulator* acc);
int64_t vr_accumulator_count(const vr_accumulator* acc);
int vr_accumulate(vr_accumulator* acc, const float* frame_rgba_device, float* out_rgba_device, void* stream);
/* Error against a reference image (ErrorMeasurePass: ErrorMeasurer.cs.slang and the reduction of
 * ErrorMeasurePass.cpp:216-250): per pixel and channel |src - ref|, squared with
 * VR_ERRM_SQUARED, (src - ref)^2 / (ref^2 + eps) with VR_ERRM_RELATIVE (relative MSE),
 * averaged over RGB with VR_ERRM_AVERAGE, zero where world_pos.w == 0 with
 * VR_ERRM_IGNORE_BACKGROUND; error_out[c] = the channel's sum over pixels / pixel count, summed
 * in FP64 in a fixed order.  diff_out (optional, device) receives the per-pixel terms.
 * Synchronises the stream. */
#define VR_ERRM_IGNORE_BACKGROUND 1
#define VR_ERRM_SQUARED 2
#define VR_ERRM_AVERAGE 4
#define VR_ERRM_RELATIVE 8
int vr_error_measure(const float* src_rgba_device, const float* ref_rgba_device, const float* world_pos_device_or_null,
                     int32_t width, int32_t height, int32_t mode, float eps, double error_out[3],
                     float* diff_out_device_or_null, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VRESTIR_H */

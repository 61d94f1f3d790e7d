/*
 * vvlic.h — C ABI of the GB300 3D line-integral-convolution (LIC) volume ray-caster.
 *
 * This is the drop-in boundary for the voLIC renderer's LIC hot path.  In the reference
 * (VectorVisualization) that path is the GLSL program composed by Renderer::loadGLSLShader
 * (renderer.cpp:807-871: inc_header.glsl + inc_lic.glsl + inc_illum.glsl + lic3d_fragment.glsl),
 * fed through the Renderer C++ API (renderer.h:28-125) and the GL uniform interface
 * (inc_header.glsl:22-63).  Every entry point below names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns a vvlic_status; nothing throws across the boundary.
 *   - Host buffers are owned by the caller; device buffers created by upload calls are owned by
 *     the context and freed by vvlic_destroy / vvlic_free_volume.
 *   - A context is bound to one CUDA device and must be used from one host thread at a time.
 *     Different contexts are independent.
 *   - `stream` arguments are cudaStream_t passed as void*; NULL means the legacy default stream.
 *   - Images are RGBA float32, row-major, row 0 = bottom row (the GL window convention),
 *     premultiplied colour exactly as the reference's gl_FragColor = dest.
 */
#ifndef VVLIC_H_
#define VVLIC_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VVLIC_ABI_VERSION 1

/* Largest streamline length per direction (stepsForward / stepsBackward). */
#define VVLIC_MAX_STEPS 256
/* Number of entries of the transfer-function tables (TransferEdit::_numEntries, transferEdit.cpp:61). */
#define VVLIC_TF_ENTRIES 256

typedef int32_t vvlic_status;
enum {
  VVLIC_OK = 0,
  VVLIC_ERR_INVALID_ARGUMENT = 1,
  VVLIC_ERR_OUT_OF_MEMORY = 2,
  VVLIC_ERR_CUDA = 3,
  VVLIC_ERR_NO_DEVICE = 4,
  VVLIC_ERR_NOT_READY = 5,     /* a required input (field, noise, TF, filter) was never set */
  VVLIC_ERR_TIMEOUT = 6,       /* a bounded device-side wait gave up */
  VVLIC_ERR_UNSUPPORTED = 7,
  VVLIC_ERR_BAD_HANDLE = 8,
  VVLIC_ERR_IO = 9,
  VVLIC_ERR_FORMAT = 10
};

/* Raw vector data types of a .raw file (reader.h DataType: DATRAW_FLOAT, DATRAW_UCHAR). */
enum { VVLIC_DTYPE_FLOAT32 = 0, VVLIC_DTYPE_UINT8 = 1 };

/* Device storage precision of the encoded field (RGBA per voxel).  The reference stores RGBA16F
 * (VectorDataSet::createTextureIterp(..., true), 3DLIC.cpp:707 -> dataset.cpp:326-331).
 * UNORM8 rounds the same float encoding to the nearest multiple of 1/255 (4 bytes per voxel). */
enum { VVLIC_STORAGE_F32 = 0, VVLIC_STORAGE_F16 = 1, VVLIC_STORAGE_BF16 = 2, VVLIC_STORAGE_UNORM8 = 3 };

/* How the kernels read the field:
 *   GATHER  - 8 texel loads per trilinear from the x-fastest RGBA array;
 *   CELL    - corner-packed cells: the 8 corners of every trilinear cell stored contiguously
 *             (8x the memory, one or two vector loads per trilinear);
 *   TEXTURE - hardware-filtered cudaTextureObjects for field and noise (8-bit fixed-point
 *             filter weights); a BF16 field's texture is a half4 copy of its BF16 texels
 *             (exact for the encoded texel values down to 2^-14);
 *   HYBRID  - field through the texture unit, noise from corner-packed cells through the
 *             load/store path, splitting the gathers over both L1 data pipes;
 *   BRICK   - field and noise texels staged per 16x8 ray tile into shared memory by TMA
 *             (cp.async.bulk.tensor), one brick pair per segment of 8 samples covering the
 *             samples' streamline reach; GATHER's arithmetic from shared memory, global memory
 *             for fetches outside the bricks.  RAYCAST renders only (no tape, no batch), static
 *             schedule; needs field rows (nx * texel bytes) and noise rows (mx * channels) that
 *             are multiples of 16 bytes (else VVLIC_ERR_UNSUPPORTED). */
enum {
  VVLIC_SAMPLER_GATHER = 0,
  VVLIC_SAMPLER_CELL = 1,
  VVLIC_SAMPLER_TEXTURE = 2,
  VVLIC_SAMPLER_HYBRID = 3,
  VVLIC_SAMPLER_BRICK = 4
};

/* Noise texture preparation (NoiseDataSet::createTexture, dataset.cpp:1176-1344).
 *   SCALAR  - noise value only (the reference without -g, read as the noise value, see quirks);
 *   SOBEL   - -g with the 3x3x3 Sobel gradients (gradient.h:37 SOBEL 1);
 *   CENTRAL - -g with the central-difference branch (gradient.cpp SOBEL 0). */
enum { VVLIC_NOISE_SCALAR = 0, VVLIC_NOISE_GRAD_SOBEL = 1, VVLIC_NOISE_GRAD_CENTRAL = 2 };

/* Streamline integrator.  HEUN is the reference's singleLICstep (inc_lic.glsl:93-145);
 * EULER and RK4 are extensions with the same step size and first-same-as-last field reuse. */
enum { VVLIC_EULER = 0, VVLIC_HEUN = 1, VVLIC_RK4 = 2 };

/* Shading model: the #define variant of inc_illum.glsl (inc_header.glsl:3-8). */
enum { VVLIC_ILLUM_NONE = 0, VVLIC_ILLUM_GRADIENT = 1, VVLIC_ILLUM_ZOECKLER = 2, VVLIC_ILLUM_MALLO = 3 };

/* Transfer-function index: lic3d_fragment.glsl:54 uses the encoded z direction (.b);
 * the slicing and vector-field shaders use the magnitude (.a). */
enum { VVLIC_TF_INDEX_DIR_Z = 0, VVLIC_TF_INDEX_MAGNITUDE = 1 };

/* Wrap mode of the 1D filter-kernel lookup: the reference sets GL_CLAMP (dataset.cpp:1499),
 * whose LINEAR filter blends the outermost taps 50% with the (zero) border colour. */
enum { VVLIC_KERNEL_CLAMP_BORDER = 0, VVLIC_KERNEL_CLAMP_EDGE = 1 };

/* Analytic filter shapes for vvlic_make_filter_table.  BOX is LICFilter::createBoxFilter
 * (dataset.cpp:1405-1413); the others stand in for the kernel PNGs the reference loads. */
enum { VVLIC_FILTER_BOX = 0, VVLIC_FILTER_TRIANGLE = 1, VVLIC_FILTER_COS2 = 2, VVLIC_FILTER_GAUSSIAN = 3 };

/* Projection of vvlic_view. */
enum { VVLIC_PERSPECTIVE = 0, VVLIC_ORTHOGRAPHIC = 1 };

/* Reproduced reference behaviours that differ from what the code evidently intends.
 *   LUMINANCE_NOISE    without gradients the noise texture is GL_LUMINANCE whose .a samples
 *                      as 1.0, so the LIC is flat (dataset.cpp:1291-1318, inc_lic.glsl:85).
 *   UNIFORM_SCALE_BUG  setRenderVolParams writes scaleInv into the scaleVol uniform and leaves
 *                      scaleVolInv at 0 whenever the shading variant uses scaleVolInv
 *                      (renderer.cpp:941-944); the light direction then ignores the sample
 *                      position.
 *   GRAD_NOISE_NO_FREQ the gradient-noise fetch freqSamplingGrad ignores freqScale
 *                      (inc_lic.glsl:61-68).
 *   ZOECKLER_LUMINANCE the Zoeckler table is a LUMINANCE_ALPHA texture (illumination.cpp:113,
 *                      172), so illumZoeckler's `.rg` reads (L, L): the specular term adds
 *                      0.9 * diffuse-table value and the stored specular alpha is never read
 *                      (inc_illum.glsl:133-145).  Off: `.g` reads the stored specular.
 * VVLIC_QUIRKS_REFERENCE is what the reference actually computes. */
enum {
  VVLIC_QUIRK_LUMINANCE_NOISE = 1u << 0,
  VVLIC_QUIRK_UNIFORM_SCALE_BUG = 1u << 1,
  VVLIC_QUIRK_GRAD_NOISE_NO_FREQ = 1u << 2,
  VVLIC_QUIRK_ZOECKLER_LUMINANCE = 1u << 3
};
#define VVLIC_QUIRKS_REFERENCE \
  (VVLIC_QUIRK_UNIFORM_SCALE_BUG | VVLIC_QUIRK_GRAD_NOISE_NO_FREQ | VVLIC_QUIRK_ZOECKLER_LUMINANCE)

/* Render parameters.  The first block is the reference's LICParams (types.h:91-109, defaults in
 * its constructor); the rest are the shader #define variants and GL state the reference sets
 * elsewhere.  Fill with vvlic_params_default() and change what you need. */
typedef struct vvlic_params {
  /* LICParams */
  float step_size_vol;    /* stepSizeVol: ray sample spacing in texture units (1/128) */
  float gradient_scale;   /* gradientScale: LIC intensity scale (30) */
  float illum_scale;      /* illumScale (1) */
  float freq_scale;       /* freqScale: noise frequency (1) */
  int32_t num_iterations; /* numIterations: bound of each of the two nested ray loops (255) */
  int32_t steps_forward;  /* stepsForward L_f (32) */
  int32_t steps_backward; /* stepsBackward L_b (32) */
  float step_size_lic;    /* stepSizeLIC h (0.01) */
  /* variants */
  int32_t integrator;     /* VVLIC_EULER / HEUN / RK4 (HEUN) */
  int32_t illum;          /* VVLIC_ILLUM_* (NONE) */
  int32_t tf_index;       /* VVLIC_TF_INDEX_* (DIR_Z) */
  int32_t speed_of_flow;  /* SPEED_OF_FLOW define: scale steps by the magnitude (0) */
  int32_t low_res;        /* Renderer::_lowRes preview overrides, renderer.cpp:947-966 (0) */
  int32_t scalar_gate;    /* freqSampling's scalar gate, inc_lic.glsl:80 (0 = off) */
  float gate_lo, gate_hi; /* gate bounds (0.1, 0.3) */
  float eye_dist_factor;  /* (logEyeDist*0.5 + 0.3) with the never-written logEyeDist = 0 (0.3) */
  float alpha_threshold;  /* early ray termination on the sample's src.a (0.95) */
  uint32_t quirks;        /* VVLIC_QUIRK_* bits (VVLIC_QUIRKS_REFERENCE) */
  /* light (GL_LIGHT0 as set up by init/updateLightPos, 3DLIC.cpp:736, renderer.cpp:431-466) */
  float light_pos[3];     /* object-space point light ((0.5, 0.5, 1.5)) */
  float spec_exp;         /* GL_SPOT_EXPONENT = Illumination specular exponent (40) */
  float light_diffuse[3]; /* (1,1,1) */
  float light_specular[3];/* (1,1,1) */
  float light_ambient[3]; /* (0,0,0) */
  /* kernel selection (no reference counterpart) */
  int32_t sampler;        /* VVLIC_SAMPLER_* (HYBRID) */
  int32_t schedule;       /* VVLIC_SCHEDULE_* (QUEUE) */
  int32_t record_tape;    /* renders record what vvlic_render_adjoint needs (0) */
  int32_t technique;      /* VVLIC_TECHNIQUE_* = the reference's RenderTechnique (RAYCAST) */
  int32_t tape_max_samples; /* recording renders: cap on the samples a ray's tape holds
                               (0 = the longest chord / spacing, which no ray exceeds).  A ray
                               with more samples than its tape sets VVLIC_CHECK_TAPE_OVERFLOW
                               and turns the adjoint's gradients to NaN. */
  int32_t reserved[3];
} vvlic_params;

/* Render technique, numbered like the reference's RenderTechnique (types.h:63-72):
 *   VOLUME    - direct volume rendering of the encoded vector field (vectorfield_fragment.glsl);
 *   RAYCAST   - the LIC ray-cast (lic3d_fragment.glsl);
 *   SLICING   - LIC on view-aligned slices (lic3d_slicing_fragment.glsl);
 *   LICVOLUME - ray-cast of a precomputed LIC volume (raycast_lic3d_fragment.glsl), see
 *               vvlic_compute_lic_volume. */
enum { VVLIC_TECHNIQUE_VOLUME = 0, VVLIC_TECHNIQUE_RAYCAST = 1, VVLIC_TECHNIQUE_SLICING = 2, VVLIC_TECHNIQUE_LICVOLUME = 3 };

/* Work distribution of a render launch:
 *   QUEUE  - persistent CTAs pull 8x4-pixel ray tiles from a device work queue, tiles ordered
 *            longest-first by their ray-box chord (no spin-waits: one atomic per tile);
 *   STATIC - one CTA per 16x8 pixel tile in raster order. */
enum { VVLIC_SCHEDULE_QUEUE = 0, VVLIC_SCHEDULE_STATIC = 1 };

/* View.  PERSPECTIVE follows Camera::setCamera (camera.cpp:56-67) followed by
 * glTranslatef(-center) (renderer.cpp:146): gluPerspective(fovy, aspect, near, far),
 * translate(pan), translate(0,0,-distance), rotate(quaternion).  ORTHOGRAPHIC (no reference
 * counterpart) casts parallel rays along `dir`; the image spans center +- right +- up in object
 * space.  Object space is the reference's: the volume is the box [0, extent] with the largest
 * physical side 1. */
typedef struct vvlic_view {
  int32_t projection;
  float quat[4];          /* camera rotation (x, y, z, w), Transform::_q; identity (0,0,0,1) */
  float distance;         /* Camera::_dist (4) */
  float pan[3];           /* Camera::_pos ((0,0,0)) */
  float fovy_deg;         /* 35 */
  float aspect;           /* <= 0: image width / height */
  float ortho_center[3];
  float ortho_right[3];
  float ortho_up[3];
  float ortho_dir[3];
} vvlic_view;

typedef struct vvlic_ctx vvlic_ctx;

/* Per-render statistics of the last render call on a context. */
typedef struct vvlic_stats {
  uint64_t samples;       /* ray samples whose LIC was computed */
  uint64_t sample_steps;  /* samples * (L_f + L_b): the throughput unit */
  uint64_t rays;          /* pixels whose ray hit the volume */
  float kernel_ms;        /* device time of the render kernel (CUDA events) */
  uint32_t check_flags;   /* VVLIC_CHECK_* bits: libraries built with VVLIC_BOUNDS_CHECK set
                             those of the out-of-range accesses the render caught (and skipped);
                             every build sets VVLIC_CHECK_TAPE_OVERFLOW after a recording render
                             or an adjoint whose tape was too short */
} vvlic_stats;

/* Index classes of the VVLIC_BOUNDS_CHECK build. */
enum {
  VVLIC_CHECK_FIELD = 1u << 0,
  VVLIC_CHECK_NOISE = 1u << 1,
  VVLIC_CHECK_SCALAR = 1u << 2,
  VVLIC_CHECK_TAPE = 1u << 3,
  VVLIC_CHECK_IMAGE = 1u << 4,
  /* a ray of the last recording render had more samples than its tape holds
     (vvlic_params.tape_max_samples): that render's adjoint gradients are NaN */
  VVLIC_CHECK_TAPE_OVERFLOW = 1u << 5,
  /* a BRICK render gave up waiting for a brick copy (or could not align its bricks) and read
     global memory instead */
  VVLIC_CHECK_BRICK = 1u << 6
};

/* ---- defaults and helpers (no device work) ------------------------------------------- */

/* LICParams() defaults (types.h:91-99) plus the reference's shader variant defaults. */
void vvlic_params_default(vvlic_params* p);
/* Camera() defaults (camera.cpp:42-47): identity rotation, distance 4, fovy 35. */
void vvlic_view_default(vvlic_view* v);
/* Human-readable name of a status code. */
const char* vvlic_status_string(vvlic_status s);
int32_t vvlic_abi_version(void);

/* Filter-kernel table of `width` uint8 texels (nextPowerTwo(width) as the reference does).
 * BOX: LICFilter::createBoxFilter (dataset.cpp:1405-1413).  TRIANGLE/COS2/GAUSSIAN are analytic
 * tables over texel centres t = (i+0.5)/W standing in for the kernel PNGs of
 * LICFilter::loadData (dataset.cpp:1416-1467).  Writes *out_width; `out` holds >= 1024 bytes. */
vvlic_status vvlic_make_filter_table(int32_t filter, int32_t width, uint8_t* out, int32_t* out_width);

/* ---- context --------------------------------------------------------------------------- */

/* Replaces Renderer::Renderer + Renderer::init (renderer.cpp:83-103) for the LIC path. */
vvlic_status vvlic_create(vvlic_ctx** ctx, int32_t device);
vvlic_status vvlic_destroy(vvlic_ctx* ctx);
/* Text of the last error on this context ("" if none).  Valid until the next call. */
const char* vvlic_last_error(const vvlic_ctx* ctx);

/* ---- inputs -------------------------------------------------------------------------- */

/* Vector field upload: VectorDataSet::loadData geometry (dataset.cpp:97-180) +
 * createTextureIterp/fillTexDataFloatInterp encoding (dataset.cpp:290-366, 533-635) +
 * Renderer::setDataTex.  `xyz` is host memory, nx*ny*nz*3 values, x fastest.
 * slice_dist may be NULL (1,1,1).  Returns a volume id for vvlic_render. */
vvlic_status vvlic_upload_field(vvlic_ctx* ctx, const void* xyz, int32_t dtype,
                                int32_t nx, int32_t ny, int32_t nz, const float* slice_dist,
                                int32_t storage, int32_t* vol_id);
/* Time-dependent field: the encoding of the linear interpolation between two timesteps at
 * t = interp_index / interp_size, as VectorDataSet::fillTexDataFloatInterp /
 * fillTexDataCharInterp compute it (dataset.cpp:533-635, 724-823) for the idle-loop animation
 * (3DLIC.cpp:129-171, checkInterpolateStage dataset.cpp:202-210).  Unlike the reference, which
 * shifts its UCHAR3 buffers by -128 in place on every call, each call starts from the raw data. */
vvlic_status vvlic_upload_field_interp(vvlic_ctx* ctx, const void* xyz0, const void* xyz1, int32_t dtype,
                                       int32_t nx, int32_t ny, int32_t nz, const float* slice_dist,
                                       int32_t storage, int32_t interp_index, int32_t interp_size,
                                       int32_t* vol_id);
/* Same from a device pointer (float32 xyz only), asynchronous on `stream`. */
vvlic_status vvlic_upload_field_device(vvlic_ctx* ctx, const float* d_xyz,
                                       int32_t nx, int32_t ny, int32_t nz, const float* slice_dist,
                                       int32_t storage, void* stream, int32_t* vol_id);
/* Replace the field of volume `vol_id` with new raw vectors of the same dimensions, in place.
 * The reference re-creates its field texture on every animation frame (idle(), 3DLIC.cpp:129-145
 * -> VectorDataSet::createTextureIterp, dataset.cpp:290-366).  Here:
 *   - the encoded texels and any cell or texture copies are rewritten without reallocation,
 *     so volume ids, the device pointers in batch job tables and captured batch graphs stay valid;
 *   - storage and slice distances stay the volume's;
 *   - a precomputed LIC volume turns stale: LICVOLUME renders return VVLIC_ERR_NOT_READY until
 *     vvlic_compute_lic_volume runs again (the reference calls updateLICVolume in that mode);
 *   - a recorded adjoint tape of this volume is dropped.
 * Waits for the device's in-flight work, then returns when the update is complete. */
vvlic_status vvlic_update_field(vvlic_ctx* ctx, int32_t vol_id, const void* xyz, int32_t dtype,
                                int32_t nx, int32_t ny, int32_t nz);
/* vvlic_update_field ordered on `stream` instead of on the host (no counterpart in the
 * reference, whose animation step idle() re-creates the texture synchronously, 3DLIC.cpp:129-145).
 * The host copy runs on the context's copy stream into a staging buffer of its own; the
 * re-encoding and layout rebuild run on `stream` after that copy and after everything already
 * enqueued on `stream`.  The call returns at once, so the copy for the next frame overlaps the
 * render of the current one.
 *   - `xyz` must stay unchanged until the copy has run (after the next operation on `stream`
 *     has completed, e.g. vvlic_synchronize).
 *   - Renders of this volume must be enqueued on `stream` too: work on other streams is not
 *     ordered against the rewrite.
 *   - Back-to-back calls are ordered among themselves: a copy waits until the previous update's
 *     encoding has consumed the staging buffer. */
vvlic_status vvlic_update_field_async(vvlic_ctx* ctx, int32_t vol_id, const void* xyz, int32_t dtype,
                                      int32_t nx, int32_t ny, int32_t nz, void* stream);
/* vvlic_update_field_async from a device array (float32 xyz, nx*ny*nz*3, x fastest) that a
 * simulation or another kernel wrote on this GPU: no host copy, no staging buffer.  The
 * re-encoding and layout rebuild run on `stream` after the work already enqueued there; `d_xyz`
 * must stay unchanged until they have run.  The same ordering rules as vvlic_update_field_async
 * hold for renders on other streams.  No counterpart in the reference (its fields come from
 * files, dataset.cpp:533-635). */
vvlic_status vvlic_update_field_device(vvlic_ctx* ctx, int32_t vol_id, const float* d_xyz, int32_t nx, int32_t ny,
                                       int32_t nz, void* stream);
/* The same with the time interpolation of vvlic_upload_field_interp. */
vvlic_status vvlic_update_field_interp(vvlic_ctx* ctx, int32_t vol_id, const void* xyz0, const void* xyz1,
                                       int32_t dtype, int32_t nx, int32_t ny, int32_t nz,
                                       int32_t interp_index, int32_t interp_size);
vvlic_status vvlic_free_volume(vvlic_ctx* ctx, int32_t vol_id);
/* Copy a volume's encoded texels (RGBA per voxel, x fastest, at the volume's storage precision:
 * 16 bytes per voxel for F32, 8 for F16/BF16) to host memory; `capacity` is the size of `out`
 * in bytes.  The texture-upload counterpart of glGetTexImage on VectorData_Tex. */
vvlic_status vvlic_download_field(vvlic_ctx* ctx, int32_t vol_id, void* out, uint64_t capacity);
/* Copy the prepared noise texels (1 or 4 bytes per voxel, see vvlic_upload_noise) to host. */
vvlic_status vvlic_download_noise(vvlic_ctx* ctx, void* out, uint64_t capacity);
/* Device bytes held by a volume (all layouts built for it). */
vvlic_status vvlic_volume_bytes(const vvlic_ctx* ctx, int32_t vol_id, uint64_t* bytes);

/* Noise upload: NoiseDataSet::createTexture (dataset.cpp:1176-1344) + Renderer::setNoiseTex.
 * `noise` is host uint8, mx*my*mz, x fastest.  mode = VVLIC_NOISE_*; gradient modes run
 * computeGradients -> filterGradients -> quantizeGradients (gradient.cpp:190-531) on the device
 * and pack RGBA = (gradient, noise) like dataset.cpp:1270-1286.  Wrap is REPEAT.  A noise of
 * the same extent and channel count as the current one is rewritten in place (texels, cell and
 * texture copies) after the device's in-flight work; any other replaces it.  Either way a
 * recorded adjoint tape is dropped. */
vvlic_status vvlic_upload_noise(vvlic_ctx* ctx, const uint8_t* noise,
                                int32_t mx, int32_t my, int32_t mz, int32_t mode);
/* vvlic_upload_noise of a noise with the current noise's extent and channel count, ordered on
 * `stream` like vvlic_update_field_async (host copy on the copy stream, gradients and layout
 * rebuild on `stream`); returns at once.  A noise of another extent returns
 * VVLIC_ERR_NOT_READY: upload it with vvlic_upload_noise first.  `noise` must stay unchanged
 * until the copy has run.  No counterpart in the reference. */
vvlic_status vvlic_upload_noise_async(vvlic_ctx* ctx, const uint8_t* noise, int32_t mx, int32_t my, int32_t mz,
                                      int32_t mode, void* stream);
/* Noise with precomputed gradients: mx*my*mz RGBA texels (quantised gradient x, y, z, noise)
 * as vvlic_upload_noise builds them; `mode` (SOBEL or CENTRAL) records their kind. */
vvlic_status vvlic_upload_noise_rgba(vvlic_ctx* ctx, const uint8_t* rgba, int32_t mx, int32_t my, int32_t mz,
                                     int32_t mode);

/* Optional secondary scalar volume for the freqSampling gate (VolumeDataSet, dataset.cpp:840-1050,
 * Renderer::setScalarTex).  Host float32, values as the shader sees them (.r). */
vvlic_status vvlic_upload_scalar(vvlic_ctx* ctx, const float* scalar,
                                 int32_t nx, int32_t ny, int32_t nz);

/* Transfer function: TransferEdit::updateTextures (transferEdit.cpp:480-543) +
 * Renderer::setTFrgbTex / setTFalphaOpacTex.  rgba: 256*4 floats (TF_RGBA, channels already
 * divided by 255 for 8-bit tables); opacity: 256 floats (the .a = opacity channel of
 * TF_AlphaOpac).  Either may be NULL to keep the current table.  Initial tables are the
 * reference default (transferEdit.cpp:76-82). */
vvlic_status vvlic_set_tf(vvlic_ctx* ctx, const float* rgba, const float* opacity);
/* The current tables (either pointer may be NULL). */
vvlic_status vvlic_get_tf(const vvlic_ctx* ctx, float* rgba, float* opacity);

/* Filter kernel: LICFilter::createTexture (dataset.cpp:1470-1500) + Renderer::setLICFilter.
 * The tap weights w[-L_b..L_f] and the inverse filter area (calcFilterKernelInvArea,
 * dataset.cpp:1503-1512) are derived at render time from the table and the current L_f/L_b. */
vvlic_status vvlic_set_filter_table(vvlic_ctx* ctx, const uint8_t* table, int32_t width,
                                    int32_t clamp_mode);
/* Explicit tap weights w[j], j = -L_b..L_f (count L_b+L_f+1), replacing the table lookup, and
 * the inverse filter area used for the intensity scale.  Pass NULL to go back to the table. */
vvlic_status vvlic_set_filter_taps(vvlic_ctx* ctx, const float* taps, int32_t steps_backward,
                                   int32_t steps_forward, float inv_filter_area);
/* The taps the next render would use (count L_b+L_f+1) and the inverse filter area. */
vvlic_status vvlic_get_filter_taps(const vvlic_ctx* ctx, float* taps, int32_t capacity,
                                   float* inv_filter_area);

/* Illuminated-streamline material: LineMat (illumination.h:38-62) and the table size of
 * Illumination (illumination.cpp:43, setTextureWidth/Height round up to a power of two).  Only
 * channel 0 of light_color / ambient / diffuse / specular enters the Zoeckler table
 * (illumination.cpp:155-160); the Mallo tables use all four. */
typedef struct vvlic_line_material {
  float light_color[4]; /* (1,1,1,1) */
  float ambient[4];     /* (0.1, ...) */
  float diffuse[4];     /* (0.5, ...) */
  float specular[4];    /* (0.8, ...) */
  float spec_exp;       /* 40 */
  float diff_exp;       /* 2 */
  int32_t width;        /* table width (256) */
  int32_t height;       /* table height (256) */
} vvlic_line_material;
void vvlic_line_material_default(vvlic_line_material* mat);
/* Rebuilds the Zoeckler and Mallo tables of Illumination::createIllumTextures
 * (illumination.cpp:58-90, 96-200, 205-290, 355-391).  The reference passes floatTex to neither
 * builder, so all three are 8-bit textures: each float is stored as round(255 * value).  The
 * initial material is the default; tables are built on first use. */
vvlic_status vvlic_set_line_material(vvlic_ctx* ctx, const vvlic_line_material* mat);
/* The three tables as the shaders sample them, RGBA8 rows of `width` texels, x fastest:
 * Zoeckler as LUMINANCE_ALPHA reads (L, L, L, A) with L = diffuse and A = 0.9 * specular;
 * Mallo diffuse and specular RGBA.  Any pointer may be NULL; width/height are always written. */
vvlic_status vvlic_get_illum_luts(vvlic_ctx* ctx, uint8_t* zoeckler, uint8_t* mallo_diffuse,
                                  uint8_t* mallo_specular, int32_t* width, int32_t* height);

/* LICParams + shader variant: Renderer::setLICParams + setRenderVolParams (renderer.cpp:925-996)
 * + the define injection of GLSLShader::loadShader (GLSLShader.cpp:120-136). */
vvlic_status vvlic_set_params(vvlic_ctx* ctx, const vvlic_params* params);
vvlic_status vvlic_get_params(const vvlic_ctx* ctx, vvlic_params* params);
/* Camera: Renderer::setCamera + Camera::setCamera (camera.cpp:56-67). */
vvlic_status vvlic_set_view(vvlic_ctx* ctx, const vvlic_view* view);

/* Per-pixel rays of the current view for volume `vol_id` at w x h, in object space:
 * origin(u,v) = c[0..2] + u*c[3..5] + v*c[6..8], direction(u,v) = c[9..11] + u*c[12..14] +
 * v*c[15..17] with u = px+0.5, v = py+0.5; c[18] = 1 when the entry parameter is clamped to
 * t >= 0 (perspective).  21 doubles are written (c[19], c[20] reserved). */
vvlic_status vvlic_view_rays(const vvlic_ctx* ctx, int32_t vol_id, int32_t w, int32_t h,
                             double* coeffs);

/* ---- rendering --------------------------------------------------------------------------- */

/* Renderer::render -> raycastVolume (renderer.cpp:126-312, 1093-1120): one LIC ray per pixel.
 * `out_rgba` is HOST memory (w*h*4 floats); the call copies the image back and synchronises. */
vvlic_status vvlic_render(vvlic_ctx* ctx, int32_t vol_id, float* out_rgba, int32_t w, int32_t h);
/* vvlic_render into HOST memory, asynchronous on `stream`: the render and the copy of the
 * image into `out_rgba` (pinned memory lets the copy overlap other work) are enqueued and the
 * call returns; the image is in `out_rgba` once `stream` has completed.  Consecutive calls
 * share one device image buffer, so they must use the same stream.  No counterpart in the
 * reference (its render draws into the window). */
vvlic_status vvlic_render_to_host_async(vvlic_ctx* ctx, int32_t vol_id, float* out_rgba, int32_t w, int32_t h,
                                        void* stream);
/* Same into DEVICE memory, asynchronous on `stream`.  `d_samples` (optional, w*h uint32) gets
 * the number of LIC samples of each ray. */
vvlic_status vvlic_render_device(vvlic_ctx* ctx, int32_t vol_id, float* d_out_rgba,
                                 int32_t w, int32_t h, uint32_t* d_samples, void* stream);
/* Adjoint of the last render (no counterpart in the reference, which has no differentiation):
 * given the image cotangent dL/d(rgba) in device memory (w*h*4 floats, the same layout as the
 * image), writes dL/dTF (256*4 RGBA entries), dL/dopacity (256) and dL/dtaps (L_b+L_f+1, the
 * explicit or table-derived tap weights) to device memory; any output pointer may be NULL.
 * The last render on this context must have been vvlic_render_device of the same volume and
 * size with params.record_tape = 1; that render recorded, per ray sample, the LIC intensity and
 * TF coordinate (with VVLIC_ILLUM_GRADIENT also the LIC gradient sum, in FP16) and, every 32
 * samples, a compositing checkpoint: 8 B (16 B lit) per sample of the longest possible ray for
 * every pixel.  Every shading model is differentiated: illumGradient through the normal, the
 * diffuse and the specular term; illumZoeckler / illumMallo through the TF colour and the
 * intensity (their table factors do not depend on TF or taps).  The TF, line material and
 * volume must not change between the recording render and this call.  Results are
 * deterministic (fixed-point accumulation); they are NaN if the tape was too short for a ray.
 * Asynchronous on `stream`. */
vvlic_status vvlic_render_adjoint(vvlic_ctx* ctx, int32_t vol_id, const float* d_dl_drgba, int32_t w, int32_t h,
                                  float* d_dl_dtf, float* d_dl_dopacity, float* d_dl_dtaps, void* stream);

/* LIC-volume precompute: Renderer::renderLICVolume (renderer.cpp:1311-1374) with
 * lic3d_volume_fragment.glsl — computeLIC * licKernel.b * gradientScale at every voxel centre of
 * an nx*ny*nz grid (the reference uses 512^3, renderer.cpp:97) with the current parameters,
 * kept with the volume (FP32; the reference's buffer is RGBA16F) for VVLIC_TECHNIQUE_LICVOLUME
 * renders.  Synchronous.  vvlic_get_stats then reports the precompute: samples = voxels,
 * sample_steps = voxels * (L_b + L_f), rays = 0 and its kernel time. */
vvlic_status vvlic_compute_lic_volume(vvlic_ctx* ctx, int32_t vol_id, int32_t nx, int32_t ny, int32_t nz);
/* Copy a volume's LIC volume (nx*ny*nz floats, x fastest) to host memory. */
vvlic_status vvlic_download_lic_volume(vvlic_ctx* ctx, int32_t vol_id, float* out, uint64_t capacity);

/* ---- batches (no reference counterpart: the reference renders one volume per frame) ---- */

/* One render job of a batch: a volume seen from a view into a device image, with its own
 * parameters and, optionally, its own filter table (else the context's filter). */
typedef struct vvlic_job {
  int32_t vol_id;
  int32_t w, h;
  float* d_out;                 /* device RGBA image, w*h*4 floats */
  vvlic_view view;
  vvlic_params params;
  const uint8_t* filter_table;  /* host table (centred in the next power of two) or NULL */
  int32_t filter_width;
  int32_t filter_clamp;
} vvlic_job;

/* Render n jobs in one persistent launch: every (job, 8x4 tile) item goes into one device work
 * queue in job-major order (jobs in submission order, each job's tiles in raster order), so the
 * warps in flight share one or two volumes' texels in cache.  All jobs must share the field storage,
 * sampler, integrator and lighting (they are compiled variants); LIC length, step sizes,
 * filter, view, image size, TF index and the other runtime parameters may differ.  The noise,
 * scalar volume and transfer function are the context's.  The launch sequence is captured in a
 * CUDA graph the first time a batch of a given shape is rendered and replayed afterwards
 * (only the job table is re-uploaded).  `stream` must not be the legacy default stream (NULL
 * selects the context's stream).  Asynchronous; vvlic_get_stats reports the batch totals. */
vvlic_status vvlic_batch_render(vvlic_ctx* ctx, const vvlic_job* jobs, int32_t n, void* stream);

/* Time the batch under each warp tile shape (8x4, 4x8, 16x2, 32x1 pixels) and each exact-noise
 * sampler (HYBRID, CELL) that the jobs' storage supports, keep the fastest for later batches of
 * this context and report it (tile width, sampler, milliseconds).  Renders the batch several
 * times.  Synchronous. */
vvlic_status vvlic_batch_autotune(vvlic_ctx* ctx, const vvlic_job* jobs, int32_t n, void* stream,
                                  int32_t* best_tile_w, int32_t* best_sampler, float* best_ms);

/* Statistics of the last render (samples are counted on the device every render). */
vvlic_status vvlic_get_stats(vvlic_ctx* ctx, vvlic_stats* stats);

/* Host watchdog (no reference counterpart; the reference blocks in SwapBuffers): wait for the
 * work queued on `stream` (and on the context's own stream) to finish, polling
 * cudaStreamQuery, for at most timeout_ms milliseconds.  VVLIC_ERR_TIMEOUT if the deadline
 * passes first; the work keeps running and a later call can wait again. */
vvlic_status vvlic_synchronize(vvlic_ctx* ctx, void* stream, int32_t timeout_ms);

/* Composite an RGBA image over an opaque white background in place:
 * background_fragment.glsl:7-20 (dest = clamp((1-dest.a)*white + dest, 0, 1)).  Host memory. */
vvlic_status vvlic_composite_background(float* rgba, int32_t w, int32_t h, const float* bg_rgba);

/* ---- on-disk formats and the image dump (host only; no context, no device) ---------- */

/* Data types of a .dat description (reader.h DataType). */
enum { VVLIC_DAT_NONE = 0, VVLIC_DAT_UCHAR = 1, VVLIC_DAT_USHORT = 2, VVLIC_DAT_FLOAT = 3 };

/* A parsed .dat volume description: DatFile::parseDatFile (reader.cpp:80-262).  Lines starting
 * with '#' are skipped; the keys ObjectFileName, Resolution, SliceThickness, Format and
 * TimeDependent are found anywhere in a line, in that order of precedence, with the value
 * after the first ':'; other lines are ignored.  Format takes UCHAR / USHORT / FLOAT and the
 * first number after it as the component count (1 if none).  raw_file is the raw-file pattern
 * (printf-style, formatted with the timestep) as written, or, when the file it names does not
 * exist, the same pattern relative to the .dat file's directory. */
typedef struct vvlic_dat_info {
  char raw_file[1024];
  int32_t resolution[3];     /* (0, 0, 0) */
  float slice_thickness[3];  /* (1, 1, 1) */
  int32_t format;            /* VVLIC_DAT_* */
  int32_t components;        /* data dimension */
  int32_t timestep_begin;    /* TimeDependent: first and last timestep (0, 0) */
  int32_t timestep_end;
} vvlic_dat_info;
/* VVLIC_ERR_IO if the .dat or a raw file of any timestep cannot be opened; VVLIC_ERR_FORMAT for
 * a key without ':' or with too few values, an unknown Format, illegal TimeDependent bounds, or
 * no ObjectFileName.  vvlic_io_error() then holds the message. */
vvlic_status vvlic_dat_parse(const char* dat_path, vvlic_dat_info* info);
/* Bytes of one timestep: type size * components * resolution product. */
uint64_t vvlic_dat_bytes(const vvlic_dat_info* info);
/* DatFile::readRawData (reader.cpp:265-303): one timestep's raw data, x fastest.  Unlike the
 * reference, which returns a partly filled buffer, a short file is VVLIC_ERR_IO. */
vvlic_status vvlic_dat_read(const vvlic_dat_info* info, int32_t timestep, void* out, uint64_t capacity);
/* VectorDataSet::loadData + createTextureIterp (dataset.cpp:96-176, 290-366): parse, check that
 * the set is a 3-component UCHAR or FLOAT field (else VVLIC_ERR_FORMAT), read `timestep` and
 * upload it with the .dat's slice thickness.  timestep < 0 takes timestep_begin. */
vvlic_status vvlic_upload_dat(vvlic_ctx* ctx, const char* dat_path, int32_t timestep, int32_t storage,
                              int32_t* vol_id);

/* NoiseDataSet::createTexture with the gradient cache (dataset.cpp:1230-1286, gradient.cpp:91-187):
 * load the noise file `path`; with gradients, take them from "<path>.grd" when that file holds
 * at least 3 bytes per voxel (the quantised x, y, z of quantizeGradients, x fastest), else
 * compute them on the device and write that file for the next time (a failed write is not an
 * error, as in the reference).  The cache does not record the gradient mode. */
vvlic_status vvlic_upload_noise_file(vvlic_ctx* ctx, const char* path, int32_t mode);

/* Noise volume file of NoiseDataSet::loadRawData (dataset.cpp:1347-1389): a 12-byte header of
 * three native int32 sizes (x, y, z) followed by x*y*z bytes, x fastest.  With out == NULL only
 * dims is written. */
vvlic_status vvlic_noise_read(const char* path, uint8_t* out, uint64_t capacity, int32_t dims[3]);
vvlic_status vvlic_noise_write(const char* path, const uint8_t* noise, const int32_t dims[3]);

/* Image dump of Renderer::saveTexture + pngWrite (renderer.cpp:340-420, imageUtils.cpp:117-139):
 * each float channel to (int)(255 * v) clamped to [0, 255], rows written top first (the image's
 * row 0 is the bottom, as GL reads it back).  VVLIC_IMAGE_PPM writes binary P6 RGB (alpha
 * dropped), VVLIC_IMAGE_PNG an 8-bit RGBA PNG.  With composite != 0 the image is first put over
 * white as background_fragment.glsl does (the window image; 0 dumps the render buffer as the
 * reference's screenshot does). */
enum { VVLIC_IMAGE_PPM = 0, VVLIC_IMAGE_PNG = 1 };
vvlic_status vvlic_image_write(const char* path, const float* rgba, int32_t w, int32_t h, int32_t kind,
                               int32_t composite);

/* pngRead (imageUtils.cpp:20-100): an 8-bit gray, gray+alpha, RGB or RGBA PNG, rows top first,
 * `channels` bytes per pixel (interlaced images: VVLIC_ERR_UNSUPPORTED).  With out == NULL only
 * w, h and channels are written. */
vvlic_status vvlic_png_read(const char* path, uint8_t* out, uint64_t capacity, int32_t* w, int32_t* h,
                            int32_t* channels);
/* LICFilter::loadData (dataset.cpp:1416-1467) + Renderer::setLICFilter: the first channel of
 * the PNG's first row becomes the filter table (centred in the next power of two, GL_CLAMP). */
vvlic_status vvlic_load_filter_png(vvlic_ctx* ctx, const char* path);
/* TransferEdit::loadTF (transferEdit.cpp:224-313) with setTFFileNames (:113-158): `name`
 * becomes "<name>_rgba.png" / "<name>_alpha.png" (or the suffixes go before the extension).
 * The first 256 pixels of the RGBA file set TF r, g, b (gray copied) and alpha (a second or
 * fourth channel).  As in the reference (`!loadRGBATF() && !loadAlphaOpacTF()`), the
 * alpha/opacity file (first channel alpha, second opacity) is read only when the RGBA file
 * cannot be. */
vvlic_status vvlic_load_tf_png(vvlic_ctx* ctx, const char* name);
/* TransferEdit::saveTF (transferEdit.cpp:163-221): 256 x 10 RGBA and gray+alpha (alpha,
 * opacity) PNGs of the current tables, each entry round(255 * v). */
vvlic_status vvlic_save_tf_png(vvlic_ctx* ctx, const char* name);

/* Message of the last failing call of this section on the calling thread. */
const char* vvlic_io_error(void);

/* ---- preprocessing on caller-owned device buffers ----------------------------------- */

/* computeGradients/filterGradients/quantizeGradients + RGBA pack (gradient.cpp:190-531,
 * dataset.cpp:1270-1286) on device buffers: d_noise (mx*my*mz uint8) -> d_rgba (4 bytes per
 * voxel: quantised gradient xyz, noise).  mode is VVLIC_NOISE_GRAD_SOBEL or _CENTRAL.
 * Allocates a temporary float gradient buffer of 12 bytes per voxel. */
vvlic_status vvlic_noise_gradients_device(const uint8_t* d_noise, int32_t mx, int32_t my,
                                          int32_t mz, int32_t mode, const float* slice_dist,
                                          uint8_t* d_rgba, void* stream);

/* ---- diagnostics (no reference counterpart) ------------------------------------------- */

/* Measured L1TEX fetch ceiling of one GPU (vvlic_measure_fetch_ceiling). */
typedef struct vvlic_fetch_ceiling {
  double tex_per_s;       /* tex3D<float4> trilinear fetches per second from an L1-resident half4 texture */
  double ld256_per_s;     /* 256-bit ld.global.nc loads per second that hit L1 */
  double group_per_s[3];  /* groups of k fetches + one 256-bit load per second, k = 1, 2, 4: the
                             fetches of one Euler, Heun and RK4 streamline step of the HYBRID
                             sampler (field through the texture unit, one noise cell load) */
  float ms[5];            /* best kernel time of each measurement (tex, ld256, k = 1, 2, 4) */
  int32_t num_sms;
  int32_t spread4;        /* lane spacing of the 8x4 lane tile the kernels use, in quarter texels */
} vvlic_fetch_ceiling;

/* Times five small kernels on `device` (about 50 ms in all; allocates and frees ~50 KB) whose
 * warps fetch like the ray-cast kernels' warps — an 8x4 lane tile `spread4` quarter texels
 * apart, advancing about a quarter texel per iteration — from data that stays in L1.  The
 * rates are the ceiling the render kernels' fetch rate is compared with (their DRAM traffic is
 * a few percent of HBM bandwidth, so HBM does not bound them). */
vvlic_status vvlic_measure_fetch_ceiling(int32_t device, int32_t spread4, vvlic_fetch_ceiling* out);

/* Largest noise (voxels) vvlic_noise_gradients_device_noalloc accepts: its fixed 16 MiB
 * gradient scratch holds four floats per voxel. */
#define VVLIC_NOALLOC_MAX_VOXELS (1u << 20)

/* No counterpart in the reference.  The same computation and output as
 * vvlic_noise_gradients_device, for callers that must not allocate device memory during the
 * call: applications that reserve their GPU memory budget at start-up and forbid later
 * allocations, or frame loops that cannot afford allocator latency and cudaFree's implicit
 * synchronisation.  The temporary gradients live in a fixed device array compiled into the
 * library (VVLIC_NOALLOC_MAX_VOXELS * 16 bytes, held on every GPU that loads the library until
 * the process exits); the caller still passes the input and output buffers.
 *   - Runs on the current CUDA device.  The first call on a device looks up that array's
 *     device address (cudaGetSymbolAddress) and caches it; make that first call before any
 *     stream capture.  The cached address does not survive cudaDeviceReset: do not call this
 *     entry point on a device after resetting it.  A call whose launch fails forgets the
 *     address, and the next call looks it up again.
 *   - mx*my*mz above VVLIC_NOALLOC_MAX_VOXELS (or an axis below 2) returns
 *     VVLIC_ERR_INVALID_ARGUMENT without launching anything.
 *   - Every call shares the array and it keeps the last call's contents; calls that overlap on
 *     the GPU (different streams or threads) race on it and must be ordered by the caller. */
vvlic_status vvlic_noise_gradients_device_noalloc(const uint8_t* d_noise, int32_t mx, int32_t my,
                                                  int32_t mz, int32_t mode, const float* slice_dist,
                                                  uint8_t* d_rgba, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* VVLIC_H_ */

/*
 * trayracer.h - C ABI of the GB300 wavefront path-tracing hot path.
 *
 * One context owns one scene, one film and the SoA wavefront buffers on one
 * CUDA device. Every entry point returns a tr_status and never exits the
 * process. Pointers are plain host or device pointers as documented per call;
 * streams are passed as opaque `void*` (a cudaStream_t, NULL = legacy default
 * stream). A context is driven by one host thread at a time.
 *
 * The per-stage entry points map 1:1 onto the stages of the reference
 * renderer (rdbruijne/trayracer):
 *   tr_generate   <- OptiX __raygen__ RayGenModes::Primary (camera rays)
 *                    Tracer/Optix/GPU/optix.cu:235-276, launched from
 *                    Tracer/Renderer/DeviceRenderer.cpp:215-218
 *   tr_extend     <- OptiX __raygen__ RayGenModes::Secondary + __closesthit__/
 *                    __miss__, Tracer/Optix/GPU/optix.cu:203-218,278-314;
 *                    for bounce 0 this is the trace half of the Primary mode
 *   tr_shade      <- Shade(RenderModes::PathTracing, DECLARE_KERNEL_PARAMS)
 *                    Tracer/CUDA/GPU/CudaFwd.h:34, Tracer/CUDA/GPU/cuda.cu:22-84,
 *                    kernel Tracer/CUDA/GPU/Shade/PathTracing.h:8-175
 *   tr_connect    <- OptiX __raygen__ RayGenModes::Shadow,
 *                    Tracer/Optix/GPU/optix.cu:316-343
 *   tr_finalize   <- FinalizeFrame, Tracer/CUDA/GPU/CudaUtilityKernels.h:27-44
 *   tr_begin_frame<- DeviceRenderer::PreRender + InitCudaCounters,
 *                    Tracer/Renderer/DeviceRenderer.cpp:137-177,
 *                    Tracer/CUDA/GPU/CudaUtilityKernels.h:6-20
 *   tr_render_frame <- DeviceRenderer::RenderFrame bounce loop,
 *                    Tracer/Renderer/DeviceRenderer.cpp:97-133
 *   tr_scene_upload <- Renderer::UpdateScene/UploadGeometry/UploadMaterials and
 *                    the SetCuda* setters, Tracer/Renderer/Renderer.cpp:79-143,
 *                    442-527, Tracer/CUDA/GPU/CudaFwd.h:9-31; the OptiX
 *                    acceleration build (Tracer/Optix/OptixRenderer.cpp:90-123,
 *                    Tracer/Resources/Model.cpp:240-306) is replaced by a host
 *                    built 8-wide BVH
 *   tr_set_camera <- DeviceRenderer::SetCamera, DeviceRenderer.cpp:25-40
 *   tr_set_settings <- KernelSettings, Tracer/Common/CommonStructs.h:145-153
 *   tr_get_statistics <- RenderStatistics::DeviceStatistics,
 *                    Tracer/Renderer/RenderStatistics.h:11-26, and RayCounters,
 *                    Tracer/Common/CommonStructs.h:208-212
 */
#ifndef TRAYRACER_H
#define TRAYRACER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TR_ABI_VERSION 3u

/* Maximum path length; the reference's DeviceRenderer::MaxTraceDepth
 * (Tracer/Renderer/DeviceRenderer.h:29). */
#define TR_MAX_DEPTH 16u

/* Largest number of paths in flight: path indices are packed in 28 bits
 * (PackedPathIxShift = 4, Tracer/Common/CommonStructs.h:46-71). */
#define TR_MAX_PATHS (1u << 28)

typedef enum tr_status {
    TR_OK = 0,
    TR_ERR_INVALID_ARGUMENT = 1,
    TR_ERR_OUT_OF_MEMORY = 2,
    TR_ERR_CUDA = 3,
    TR_ERR_NO_SCENE = 4,
    TR_ERR_NOT_READY = 5,
    TR_ERR_LIMIT = 6,
    TR_ERR_DEVICE_FAULT = 7
} tr_status;

/* Closure (BSDF) per material. The reference selects its closure by commenting
 * code in Tracer/CUDA/GPU/Shade/PathTracing.h:127-129 (Lambert live); here it
 * is a material property. */
typedef enum tr_closure {
    TR_CLOSURE_LAMBERT = 0, /* Shade/BSDF/Lambert.h:53-59 */
    TR_CLOSURE_DIFFUSE = 1, /* Shade/BSDF/Diffuse.h:36-42 */
    TR_CLOSURE_DISNEY = 2   /* Shade/BSDF/Disney.h:573-579 */
} tr_closure;

/* Kernel setting flags. */
enum {
    /* Reproduce the reference's sampling exactly: TEA/LCG random streams
     * (thirdparty/CUDA/random.h:31-67, seeded as in optix.cu:247 and
     * PathTracing.h:103), binary-search light pick over the exclusive energy
     * prefix (CudaLights.h:38-59) with LightEnergy = last prefix
     * (Renderer.cpp:500), three independent light barycentrics
     * (CudaLights.h:107-108), its emissive-hit weighting (PathTracing.h:76-97),
     * its Disney lobe-sample reuse of r0 (Disney.h:491-521) and its NEE gate
     * (CudaLights.h:118). Without this flag the path uses the counter-based
     * RNG, an alias-table light pick, uniform triangle points, balance-
     * heuristic MIS on emissive hits and a rescaled lobe sample. */
    TR_FLAG_REFERENCE_SAMPLING = 1u << 0,
    /* Write the first-hit albedo and normal guide buffers
     * (PathTracing.h:48-52,66-70,93-97). */
    TR_FLAG_WRITE_AOVS = 1u << 1,
    /* With TR_FLAG_REFERENCE_SAMPLING: take the random numbers that the
     * reference draws as arguments of one call (camera jitter optix.cu:147,
     * lens sample optix.cu:55, light barycentrics CudaLights.h:107, closure
     * r0/r1 PathTracing.h:129) right to left instead of left to right. C++
     * leaves that order unspecified; right to left is what the g++ host build
     * of the reference does. */
    TR_FLAG_REFERENCE_DRAW_RTL = 1u << 2,
    /* Count the BVH nodes visited and triangles tested by the extend and
     * connect launches (tr_statistics.traversal_*). Adds atomics; for
     * measurement runs outside timed regions. */
    TR_FLAG_COUNT_TRAVERSAL = 1u << 3
};

/* ≙ KernelSettings (Tracer/Common/CommonStructs.h:145-153) plus the knobs the
 * reference hard-wires. */
typedef struct tr_kernel_settings {
    uint32_t multi_sample;   /* samples per pixel in one frame (paths in flight = W*H*multi_sample) */
    uint32_t max_depth;      /* bounces per path, <= TR_MAX_DEPTH */
    uint32_t seed;           /* frame seed */
    float ray_epsilon;       /* tmin of every ray, shadow tmax = dist - 2*eps */
    uint32_t rr_start;       /* first path length with Russian roulette (reference: 1); >= max_depth disables */
    uint32_t flags;          /* TR_FLAG_* */
    float max_color;         /* firefly clamp of SafeColor (CudaUtility.h:91); <= 0 selects 10 */
    uint32_t traversal_step_limit; /* bound on the BVH node visits of one ray's traversal; 0 selects 2^22.
                                      A ray that runs out ends with the hit found so far and sets
                                      tr_statistics.device_error (the reference has no bound: OptiX
                                      traversal is opaque) */
} tr_kernel_settings;

/* ≙ the camera fields of LaunchParams (Tracer/Common/CommonStructs.h:170-184). */
typedef struct tr_camera {
    float position[3];
    float side[3];
    float up[3];
    float forward[3];
    float aperture;
    float distortion;
    float focal_dist;
    float fov;              /* radians */
    int32_t bokeh_side_count;
    float bokeh_rotation;
} tr_camera;

/* One material with constant properties (the reference's 13 material
 * properties, Tracer/Common/CommonStructs.h:78-93; values are rounded to fp16
 * on upload as Material::Property::Build does, Material.cpp:56-78). */
typedef struct tr_material_desc {
    float diffuse[3];
    float emissive[3];
    float metallic;
    float subsurface;
    float specular;
    float roughness;
    float specular_tint;
    float anisotropic;
    float sheen;
    float sheen_tint;
    float clearcoat;
    float clearcoat_gloss;
    uint32_t closure;       /* tr_closure */
} tr_material_desc;

/* One triangle mesh (≙ Model, Tracer/Resources/Model.h). Normals and
 * texcoords are per vertex and optional (NULL: face normal / zero uv). */
typedef struct tr_mesh_desc {
    const float* positions;        /* float3 x vertex_count */
    const float* normals;          /* float3 x vertex_count or NULL */
    const float* texcoords;        /* float2 x vertex_count or NULL */
    uint32_t vertex_count;
    uint32_t triangle_count;
    const uint32_t* indices;       /* uint3 x triangle_count */
    const uint32_t* material_indices; /* triangle_count entries into the scene material list */
} tr_mesh_desc;

/* One placement of a mesh (≙ Instance: OptixInstance::transform, instanceId;
 * Tracer/Resources/Instance.cpp:39-49). */
typedef struct tr_instance_desc {
    uint32_t mesh;                 /* index into tr_scene_desc.meshes */
    uint32_t reserved;
    float transform[12];           /* object -> world, 3 rows (r.x, r.y, r.z, t) as OptixInstance::transform */
} tr_instance_desc;

/* Material property slots (≙ MaterialPropertyIds, CommonStructs.h:78-96), the
 * order of tr_scene_desc.material_textures. */
enum {
    TR_PROP_ANISOTROPIC = 0,
    TR_PROP_CLEARCOAT = 1,
    TR_PROP_CLEARCOAT_GLOSS = 2,
    TR_PROP_DIFFUSE = 3,
    TR_PROP_EMISSIVE = 4,       /* takes no texture (Material.cpp: Emissive is colour only) */
    TR_PROP_METALLIC = 5,
    TR_PROP_NORMAL = 6,         /* texture only: a normal map */
    TR_PROP_ROUGHNESS = 7,
    TR_PROP_SHEEN = 8,
    TR_PROP_SHEEN_TINT = 9,
    TR_PROP_SPECULAR = 10,
    TR_PROP_SPECULAR_TINT = 11,
    TR_PROP_SUBSURFACE = 12,
    TR_PROP_COUNT = 13
};
#define TR_NO_TEXTURE 0xFFFFFFFFu

/* ≙ Texture (Tracer/Resources/Texture.cpp:83-139): width x height RGBA texels
 * as IEEE binary16 bits, row by row, sampled as the reference's texture
 * objects are (bilinear filtering, wrap addressing, normalised coordinates).
 * A property with a texture is its colour times the texture's RGB at the hit's
 * texture coordinate (GetColor, CudaMaterial.h:77-95). */
typedef struct tr_texture_desc {
    uint32_t width;
    uint32_t height;
    const uint16_t* texels;        /* 4 x width x height */
} tr_texture_desc;

typedef struct tr_scene_desc {
    const tr_mesh_desc* mesh;      /* one mesh, one identity instance (when instance_count == 0) */
    const tr_material_desc* materials;
    uint32_t material_count;
    uint32_t bvh_leaf_size;        /* 1..3 triangles per leaf, 0 = default (3) */
    uint32_t build_threads;        /* host threads for the BVH build, 0 = all */
    uint32_t instance_count;       /* > 0: two-level scene, instances[] place meshes[] */
    /* two-level scenes (≙ Scene::Instances / Models, Renderer::UploadGeometry,
     * Renderer.cpp:442-505): one BVH per mesh, one over the instances */
    const tr_mesh_desc* meshes;
    const uint32_t* mesh_material_offsets; /* per mesh, added to its material indices (≙ MaterialOffsets); NULL = 0 */
    const tr_instance_desc* instances;
    uint32_t mesh_count;
    uint32_t texture_count;
    const tr_texture_desc* textures;
    const uint32_t* material_textures; /* material_count x TR_PROP_COUNT texture indices or TR_NO_TEXTURE; NULL = none */
} tr_scene_desc;

typedef struct tr_config {
    int32_t device;                /* CUDA device ordinal */
    uint32_t abi_version;          /* TR_ABI_VERSION */
} tr_config;

/* ≙ RenderStatistics::DeviceStatistics (RenderStatistics.h:11-26) + per-stage
 * device times of the last frame, measured with CUDA events on the stream the
 * frame was rendered on. */
typedef struct tr_statistics {
    uint64_t path_count;            /* extend + shadow rays of the last frame */
    uint64_t primary_path_count;
    uint64_t secondary_path_count;
    uint64_t deep_path_count;
    uint64_t shadow_ray_count;
    uint32_t extend_rays[TR_MAX_DEPTH]; /* queue length per bounce */
    uint32_t shadow_rays[TR_MAX_DEPTH];
    float render_time_ms;
    float generate_time_ms;
    float extend_time_ms;
    float shade_time_ms;
    float connect_time_ms;
    float finalize_time_ms;
    uint32_t sample_count;          /* accumulated samples per pixel */
    uint32_t device_error;          /* nonzero: a kernel recorded a bounded-loop overrun (traversal stack
                                       depth or traversal_step_limit) since the last tr_reset */
    /* with TR_FLAG_COUNT_TRAVERSAL, summed over the frames since tr_reset */
    uint64_t traversal_extend_nodes;
    uint64_t traversal_extend_tris;
    uint64_t traversal_connect_nodes;
    uint64_t traversal_connect_tris;
    uint32_t hit_rays[TR_MAX_DEPTH];    /* extend rays per bounce that hit something */
    /* with TR_FLAG_COUNT_TRAVERSAL, summed over the frames since tr_reset: path radiance
     * read-modify-writes by shade (emissive hits) and by connect (unoccluded shadow rays) */
    uint64_t radiance_updates_shade;
    uint64_t radiance_updates_connect;
    uint32_t iterations;            /* after tr_render_samples: continuous-wavefront iterations that traced rays */
    uint32_t launches;              /* after tr_render_samples: kernels of that render */
    uint64_t hit_ray_count;         /* extend rays that hit something (the sum of hit_rays) */
} tr_statistics;

/* Scene numbers: triangle/light/BVH sizes and the host build time. */
typedef struct tr_scene_info {
    uint32_t triangle_count;
    uint32_t light_count;
    uint32_t material_count;
    uint32_t bvh_node_count;        /* 8-wide nodes (208 B with fp32 child boxes, 80 B quantized) */
    uint64_t device_bytes;          /* scene bytes resident on the device */
    float light_energy;             /* total emitted energy used for light picks */
    float build_time_ms;            /* host flattening + BVH build */
    float upload_time_ms;
    float scene_bounds[6];
} tr_scene_info;

/* Device pointers of the wavefront buffers (plane-major SoA), for parity
 * dumps and external consumers. `capacity` is the plane stride in elements.
 *   path_state[k]: 3 planes of float4: (O.xyz, bits(pathIx<<4|flags)),
 *                  (D.xyz, bits(packed normal)), (T.xyz, extend pdf).
 *                  k = 0: the extend queue (written by tr_generate and
 *                  tr_shade, read by tr_extend); k = 1: the hit queue (the
 *                  extend queue's rays that hit something, in no particular
 *                  order, written by tr_extend, read by tr_shade).
 *   hits:          uint4 per hit-queue slot: (bary 16:16, instIx, primIx, bits(t)).
 *   shadow:        3 planes of float4: (O.xyz, bits(pathIx)), (L.xyz, dist),
 *                  (T.xyz, 0).
 *   radiance:      float4 per path index (sum of this frame's contributions).
 *   accumulator:   float4 per pixel (sum over frames, .w = sample count).
 *   counters:      uint32[5*(TR_MAX_DEPTH+1)+1], 17 words per group: extend
 *                  queue length per bounce, shadow queue length per bounce,
 *                  the work cursors of the extend and connect launches, the
 *                  hit queue length per bounce; then the path cursor of
 *                  tr_adjoint_frame. */
typedef struct tr_buffers {
    void* path_state[2];
    void* hits;
    void* shadow;
    void* radiance;
    void* accumulator;
    void* albedo;
    void* normals;
    void* colors;
    void* counters;
    uint64_t capacity;
    uint32_t width;
    uint32_t height;
} tr_buffers;

/* Launch and build parameters chosen by tr_autotune (0 = default). */
typedef struct tr_tuning {
    uint32_t bvh_leaf_size;         /* triangles per BVH leaf, 1..3 (BVH rebuilt from the kept host copy) */
    uint32_t refill_below;          /* persistent traversal warps take new rays below this many active lanes, 1..32 */
    uint32_t extend_blocks_per_sm;  /* persistent extend grid, 1..occupancy */
    uint32_t connect_blocks_per_sm; /* persistent connect grid, 1..occupancy */
    uint32_t shade_waves;           /* shade grid cap in waves of resident blocks, 1..64 */
    uint32_t sort_hits;             /* 1: counting sort of each bounce's hits by material before shade */
    uint32_t traversal_threads;     /* threads per block of the extend / connect launches: 64 or 128 */
    uint32_t shade_threads;         /* threads per block of the shade launches: 64 or 128 */
    uint32_t bvh_nodes;             /* node layout: 0 auto (fp32 child boxes while the nodes fit 64 MB and
                                       the scene has one level, else 8-bit quantized), 1 fp32 (208 B a
                                       node), 2 quantized (80 B); tr_get_tuning reports the layout in use
                                       (1 or 2) */
} tr_tuning;

typedef struct tr_tune_report {
    tr_tuning chosen;
    float frame_ms_default;         /* one frame with the default tuning */
    float frame_ms_tuned;           /* one frame with the chosen tuning */
    uint32_t trials;                /* configurations timed */
    uint32_t reserved;
} tr_tune_report;

/* ---- lifetime ---- */
tr_status tr_create(const tr_config* config, void** out_ctx);
tr_status tr_destroy(void* ctx);
const char* tr_status_string(tr_status status);
const char* tr_last_error(void* ctx);

/* ---- scene / camera / settings ---- */
tr_status tr_scene_upload(void* ctx, const tr_scene_desc* scene);
tr_status tr_get_scene_info(void* ctx, tr_scene_info* info);
/* Replaces the material table of the uploaded scene (same count) without
 * rebuilding the BVH; emissive materials may change radiance but the set of
 * emissive triangles must stay the same (light records and the alias table
 * are rebuilt). Resets the accumulation. No reference counterpart: the
 * reference re-uploads changed materials through Renderer::UpdateScene
 * (Renderer.cpp:79-143). */
tr_status tr_update_materials(void* ctx, const tr_material_desc* materials, uint32_t count);
tr_status tr_set_camera(void* ctx, const tr_camera* camera);
tr_status tr_set_settings(void* ctx, const tr_kernel_settings* settings);
tr_status tr_resize(void* ctx, uint32_t width, uint32_t height);
tr_status tr_reset(void* ctx);

/* ---- per-stage wavefront interface ---- */
tr_status tr_begin_frame(void* ctx, void* stream);
tr_status tr_generate(void* ctx, void* stream);
tr_status tr_extend(void* ctx, void* stream, uint32_t bounce);
tr_status tr_shade(void* ctx, void* stream, uint32_t bounce);
tr_status tr_connect(void* ctx, void* stream, uint32_t bounce);
tr_status tr_finalize(void* ctx, void* stream);

/* Whole frame: begin, generate, max_depth x (extend, shade, connect),
 * finalize. The bounce loop runs from device-side queue counters without host
 * round trips; with use_graph != 0 it is captured once per configuration into
 * a CUDA graph and replayed. */
tr_status tr_render_frame(void* ctx, void* stream, int32_t use_graph);

/* spp samples per pixel (a multiple of multi_sample) added to the
 * accumulation, as spp / multi_sample calls of tr_render_frame would add them
 * (the same sample keys), but rendered as one continuous wavefront: the
 * frame's width * height * multi_sample path slots are kept full from a device
 * sample cursor, each path regenerated with the next sample as soon as it
 * ends, so the frames' late bounces do not leave the GPU idle between frames;
 * with use_graph the iterations run as a CUDA graph while loop. The image
 * equals the frame sequence's up to the order of the per-pixel sums (all spp
 * samples summed in sample order, not frame by frame). Allocates 16 B per
 * sample for the per-sample radiance. Where the continuous kernels do not
 * apply (TR_FLAG_REFERENCE_SAMPLING, TR_FLAG_WRITE_AOVS, other render modes,
 * more than 2^30 samples) it renders the frames. After
 * it, tr_get_statistics reports totals: path_count, shadow_ray_count,
 * hit_ray_count, primary_path_count (width * height * spp) and
 * secondary_path_count (every other extend ray), iterations and launches;
 * the per-bounce arrays are zero. An eager render (use_graph = 0) also
 * reports its stage times, summed over the iterations: generate_time_ms the
 * plan kernels, extend_time_ms (with the camera rays of new samples),
 * shade_time_ms, connect_time_ms, finalize_time_ms the round starts,
 * finalize and sample-count advance. Replaces n accumulating frames of the
 * reference's application loop (Tracer/App/RunApp.cpp:144, one
 * DeviceRenderer::RenderFrame per displayed frame,
 * Tracer/Renderer/DeviceRenderer.cpp:97-133). */
tr_status tr_render_samples(void* ctx, void* stream, uint32_t spp, int32_t use_graph);

/* Path-replay adjoint (Vicini, Speierer, Jakob, SIGGRAPH 2021) of the last
 * rendered frame: adds to param_grad (device, material_count x 9 floats:
 * d/d base colour r, g, b, roughness, metallic, specular, emission r, g, b)
 * the gradient of a loss whose derivative with respect to each path's
 * radiance is scale * pixel_grad[pixel] (device, float4 per pixel; for an
 * image averaged over S samples per pixel pass scale = 1/S). Paths are
 * replayed from their random keys (rays re-traced, nothing stored per
 * vertex); sampled directions, pdfs and MIS weights are held fixed.
 * Default sampling mode only. No reference counterpart (the reference does
 * not differentiate). */
tr_status tr_adjoint_frame(void* ctx, void* stream, const float* pixel_grad, float scale, float* param_grad);

/* One frame (as tr_render_frame without a graph) into caller-owned device
 * buffers, allocating no device memory: for callers that cannot allocate
 * where they render (a render loop that must not stall the device on
 * cudaMalloc/cudaFree, a host that owns all device memory through its own
 * pool). No counterpart in the reference. The frame's scratch (path queues,
 * hits, per-path radiance, counters) lives in one file-scope device array of
 * the library (about 22 MiB, held by every GPU that loads the library until
 * exit), so width * height * multi_sample must not exceed 131072 paths
 * (TR_ERR_LIMIT otherwise). accumulator (float4 per pixel) is read unless
 * sample_count is 0 and written; colors (float4 per pixel) = accumulator /
 * (sample_count + multi_sample). The scene, camera, settings and resolution
 * come from the context (set up beforehand; tr_scene_upload allocates). The
 * first call on a device looks up the array's device address (which loads the
 * library's device image there); make that first call before any stream
 * capture. The address is kept for the life of the process and does not
 * survive a cudaDeviceReset of that device. Every call shares the array and
 * rewrites what it must start from: calls that overlap on the GPU (other
 * streams, other threads, other contexts) race. Guide buffers
 * (TR_FLAG_WRITE_AOVS) are not written. The path-tracing render mode only
 * (TR_ERR_INVALID_ARGUMENT after tr_set_render_mode to another mode). The
 * launch shapes are the context's tuning (tr_set_tuning / tr_autotune) without
 * the hit sort. tr_get_statistics after this call reports this frame (ray
 * counts, device_error) from the shared array, so a call that overlaps it
 * races with that read too. The calling thread's current device is restored
 * on return. */
tr_status tr_render_frame_noalloc(void* ctx, void* stream, float* accumulator, float* colors, uint32_t sample_count);

/* ---- render modes ----
 * ≙ the renderMode / renderFlags arguments of DeviceRenderer::RenderFrame
 * (DeviceRenderer.cpp:97-106) and KernelSettings::aoDist / zDepthMax: mode is a
 * RenderModes value (CommonStructs.h:110-125: 0 AmbientOcclusion,
 * 1 AmbientOcclusionShading, 2 Bitangent, 3 GeometricNormal, 4 MaterialID,
 * 5 MaterialProperty, 6 ObjectID, 7 PathTracing (default), 8 ShadingNormal,
 * 9 Tangent, 10 TextureCoordinate, 11 Wireframe, 12 ZDepth); flags selects the
 * MaterialPropertyIds value of mode 5. Modes other than 7 run the reference's
 * other shade kernels (Tracer/CUDA/GPU/Shade/*.h) through tr_render_frame; the
 * per-stage entries accept mode 7 only. Changing the mode resets the
 * accumulation. */
tr_status tr_set_render_mode(void* ctx, uint32_t mode, uint32_t flags, float ao_dist, float z_depth_max);

/* ---- sky ----
 * ≙ Tracer::Sky (Tracer/Renderer/Sky.h:16-67, Sky.cpp): the Preetham sky that a
 * path sees when it leaves the scene (SampleSky, CudaSky.h:105-156, called by
 * PathTracing.h:40-55). A context starts with the sky disabled (misses are
 * black); the reference's Scene starts with Sky's defaults (enabled, sun
 * straight up, 32 arc minutes, intensity 1000, turbidity 4, bias 1). */
typedef struct tr_sky_desc {
    uint32_t enabled;
    uint32_t draw_sun;            /* the sun disc is seen by camera and specular paths */
    float sun_dir[3];             /* normalised on set (Sky::SetSunDir) */
    float sun_angular_diameter;   /* arc minutes */
    float sun_intensity;
    float turbidity;              /* clamped to [1, 10] (Sky::SetTurbidity) */
    float selection_bias;         /* Sky::SetSelectionBias: scales the sun's NEE energy */
} tr_sky_desc;

/* Sets (or with sky = NULL disables) the sky; resets the accumulation. */
tr_status tr_set_sky(void* ctx, const tr_sky_desc* sky);

/* ---- scene files ----
 * ≙ SceneFile::Load (Tracer/FileIO/SceneFile.cpp:89-441, 683-730) with
 * ModelFile::Import / TextureFile::Import (ModelFile.cpp:53-160, 331-449,
 * TextureFile.cpp:33-175): the reference's scene JSON ("models", "instances",
 * "materials", "camera", "renderer", "sky"; "post" is ignored) read into a
 * two-level tr_scene_desc. Models load from the reference's model cache format
 * ("MDL" version 2: the file itself, or the cache file the reference keeps for
 * it, cache/<hash of its path>.bin) or from Wavefront OBJ; textures from the
 * reference's texture cache format ("TEX" version 2, likewise). Relative paths
 * resolve against base_dir (NULL: the current directory, as the reference
 * resolves them). Meshes are ordered by first use among the instances and
 * materials concatenated per mesh, as Renderer::BuildMaterials orders them;
 * every material takes TR_CLOSURE_LAMBERT, the closure the reference shades
 * with. */
typedef struct tr_scene_file_info {
    const tr_scene_desc* scene;     /* NULL when the file places no instance */
    tr_camera camera;               /* "camera" (CameraNode defaults when absent) */
    float camera_target[3];
    float camera_up[3];
    tr_kernel_settings settings;    /* "renderer" over Renderer::DefaultSettings (flags 0) */
    float ao_dist;
    float z_depth_max;
    tr_sky_desc sky;                /* "sky" over Sky's defaults (enabled) */
    uint32_t mesh_count;
    uint32_t instance_count;
    const char* const* mesh_names;      /* model name per mesh */
    const char* const* instance_names;  /* per instance */
    const char* const* material_names;  /* per material */
    const char* warnings;           /* one line per model or texture that could not be read ("" if none);
                                       as in the reference, their instances or textures are left out */
} tr_scene_file_info;

/* Loads a scene file; *out_file owns every array the info points at. */
tr_status tr_scene_file_load(const char* path, const char* base_dir, void** out_file);
tr_status tr_scene_file_get_info(void* file, tr_scene_file_info* out);
tr_status tr_scene_file_free(void* file);
/* Message of the last failed scene-file or cache call on this thread. */
const char* tr_scene_file_last_error(void);

/* ≙ SaveToCache of ModelFile.cpp:53-95: writes a mesh and its materials in
 * the reference's model cache format (a mesh without normals gets smooth
 * vertex normals, as the reference's importer generates them; without
 * texcoords, zeros). material_names: material_count names;
 * texture_paths: NULL or material_count x TR_PROP_COUNT paths (NULL or "" for
 * none) stored with the texture-enabled properties. */
tr_status tr_model_cache_write(const char* path, const tr_mesh_desc* mesh, const tr_material_desc* materials,
                               const char* const* material_names, const char* const* texture_paths,
                               uint32_t material_count);
/* ≙ SaveToCache of TextureFile.cpp:33-48: RGBA binary16 texels. */
tr_status tr_texture_cache_write(const char* path, uint32_t width, uint32_t height, const uint16_t* texels);

/* ---- ray pick ----
 * ≙ RayPickResult (CommonStructs.h:132-141): the camera position, the direction
 * of the picked pixel's camera ray, and what the ray hit first (instance and
 * mesh-local triangle, ~0u both on a miss; tmax = the hit distance, 1e30 on a
 * miss). */
typedef struct tr_ray_pick_result {
    float ray_origin[3];
    uint32_t inst_ix;
    float ray_dir[3];
    uint32_t prim_ix;
    float tmax;
} tr_ray_pick_result;

/* ≙ DeviceRenderer::PickRay (DeviceRenderer.cpp:71-92) with the RayPick raygen
 * (optix.cu:345-377): one camera ray through pixel (x, y) counted from the top
 * row (the ray takes row height - y, as the reference does), random stream
 * seeded 0, closest hit with the scene's ray epsilon. Runs on stream and waits
 * for it; any pixel coordinates are accepted (outside the image the ray leaves
 * the frustum). Needs a scene, a camera and a resolution. */
tr_status tr_pick_ray(void* ctx, void* stream, int32_t x, int32_t y, tr_ray_pick_result* out);

/* ---- tuning ----
 * No counterpart in the reference (OptiX picks its own launch shapes). */
#define TR_TUNE_SKIP_BVH (1u << 0)  /* tr_autotune: keep the BVH leaf size */
#define TR_TUNE_SAMPLES (1u << 1)   /* tr_autotune: time continuous renders (tr_render_samples of
                                       4 x multi_sample samples per pixel) instead of frames */
/* Current tuning (after the first frame: the launch shapes in use). */
tr_status tr_get_tuning(void* ctx, tr_tuning* tuning);
/* Applies a tuning; a new bvh_leaf_size rebuilds the BVH from the host copy of
 * the mesh kept since tr_scene_upload. Zero fields take the defaults. */
tr_status tr_set_tuning(void* ctx, const tr_tuning* tuning);
/* Times graph-replayed frames of the current scene, camera, settings and
 * resolution (one warm-up + two timed frames per configuration; with
 * TR_TUNE_SAMPLES one warm-up + one timed continuous render of 4 x
 * multi_sample samples per pixel, and no material sort, which the continuous
 * kernels do not use) over the block sizes of the traversal and shade
 * launches, the lane refill threshold, the persistent extend / connect grids,
 * the shade grid cap, the material sort of the hits and (unless
 * TR_TUNE_SKIP_BVH) the BVH leaf size, one parameter at a time, keeps the
 * fastest and resets the accumulation. The report's frame_ms_* are per frame,
 * or per continuous render with TR_TUNE_SAMPLES. */
tr_status tr_autotune(void* ctx, void* stream, uint32_t flags, tr_tune_report* report);

/* ---- batched rendering ----
 * Many independent scenes of uneven triangle count, resolution and sample
 * count rendered by one continuous wavefront. No counterpart in the reference
 * (one DeviceRenderer renders one scene with a host bounce loop,
 * Tracer/Renderer/DeviceRenderer.cpp:97-133); the per-stage kernels are the
 * ones behind tr_extend / tr_shade / tr_connect. Each item's scene gets its
 * own BVH; the buffers are concatenated on the device. All items' samples are
 * fed from a device cursor into a pool of pool_paths path slots (0: 2^25):
 * every iteration traces the paths carried over from the last one and starts
 * new samples in the slots that finished paths left, so the pool stays full
 * until the last samples drain. With use_graph the iterations run as a CUDA
 * graph while loop whose condition the device sets. A path's random numbers
 * are keyed as in tr_render_frame (pixel, sample, bounce, seed) and each
 * pixel's samples are summed in sample order, so every item renders the image
 * tr_render_frame gives for that scene with multi_sample = spp from a reset
 * accumulator (to a few ulps: the batch kernels are separate instances the
 * compiler may contract differently). */
typedef struct tr_batch_item {
    const tr_scene_desc* scene;     /* read during tr_batch_create only */
    tr_camera camera;
    uint32_t width;
    uint32_t height;
    uint32_t spp;                   /* samples per pixel of one tr_batch_render */
    uint32_t reserved;
} tr_batch_item;

typedef struct tr_batch_info {
    uint32_t item_count;
    uint32_t round_count;           /* item ranges that share the per-sample radiance buffer (2^30 samples) */
    uint64_t path_count;            /* sum of width * height * spp */
    uint64_t pixel_count;           /* sum of width * height */
    uint64_t triangle_count;
    uint64_t device_bytes;
    uint32_t pool_paths;            /* path slots of the wavefront */
    uint32_t reserved;
    float build_time_ms;            /* host flattening + BVH builds */
    float upload_time_ms;
} tr_batch_info;

typedef struct tr_batch_statistics {
    uint64_t extend_rays;           /* over all iterations of the last render */
    uint64_t shadow_rays;
    uint64_t hit_rays;
    float render_time_ms;           /* CUDA events around the last render */
    uint32_t device_error;
    uint64_t traversal_extend_nodes; /* with TR_FLAG_COUNT_TRAVERSAL */
    uint64_t traversal_extend_tris;
    uint64_t traversal_connect_nodes;
    uint64_t traversal_connect_tris;
    uint32_t iterations;            /* wavefront iterations that traced rays */
    uint32_t launches;              /* kernels of the last render (4 per iteration, per round 1 + 4) */
} tr_batch_statistics;

/* Builds and uploads all items (host threads build the BVHs). Items are
 * one-mesh scenes (instance_count 0), with or without textures (the batch
 * owns a copy of each item's textures). Device memory: 160 B per path slot,
 * 16 B per sample of the largest round, 32 B per pixel. TR_ERR_LIMIT when an
 * item has more than 2^30 samples, pool_paths >= 2^28 or count >= 2^24. */
tr_status tr_batch_create(const tr_config* config, const tr_batch_item* items, uint32_t count, uint64_t pool_paths,
                          void** out_batch);
tr_status tr_batch_destroy(void* batch);
const char* tr_batch_last_error(void* batch);
tr_status tr_batch_get_info(void* batch, tr_batch_info* info);
/* Renders every item's spp samples from a zeroed accumulator. settings:
 * max_depth, seed, ray_epsilon, rr_start, max_color as for tr_set_settings;
 * multi_sample is ignored; TR_FLAG_REFERENCE_SAMPLING, TR_FLAG_WRITE_AOVS and
 * TR_FLAG_REFERENCE_DRAW_RTL are rejected. use_graph: one CUDA graph (a while
 * loop per round), captured again when the settings change; without it the
 * host runs the iterations, reading the queue length back after each. */
tr_status tr_batch_render(void* batch, void* stream, const tr_kernel_settings* settings, int32_t use_graph);
tr_status tr_batch_get_statistics(void* batch, tr_batch_statistics* stats);
/* Device pointer to an item's colors (float4 per pixel, row-major). */
tr_status tr_batch_get_colors(void* batch, uint32_t item, void** device_rgba);
/* Copies an item's colors to host memory (bytes >= width * height * 16). */
tr_status tr_batch_download(void* batch, void* stream, uint32_t item, float* host_rgba, uint64_t bytes);

/* ---- results ---- */
tr_status tr_synchronize(void* ctx, void* stream);
tr_status tr_get_statistics(void* ctx, tr_statistics* stats);
tr_status tr_get_buffers(void* ctx, tr_buffers* buffers);
/* Copy the finalized colors (float4 per pixel) to host memory. */
tr_status tr_download_image(void* ctx, void* stream, float* host_rgba, uint64_t bytes);
/* Copy the accumulator (float4 per pixel) to host memory. */
tr_status tr_download_accumulator(void* ctx, void* stream, float* host_rgba, uint64_t bytes);

/* Synchronous copies between host memory and device memory of this
 * context's device (e.g. the buffers of tr_get_buffers), for inspection and
 * for injecting stage inputs. */
tr_status tr_copy_from_device(void* ctx, void* host_dst, const void* device_src, uint64_t bytes);
tr_status tr_copy_to_device(void* ctx, void* device_dst, const void* host_src, uint64_t bytes);

/* Host-side check of the acceleration structure: builds the 8-wide BVH of
 * `scene` on the host and traverses n rays (float4 O, float4 D) with the
 * traversal source of tr_extend / tr_connect compiled for the CPU.
 * any_hit bit 0 clear: closest hit over [tmin, 1e30], hits as tr_extend writes
 * them (uint4: bary 16:16, instIx, primIx, bits(t)); set: first hit over
 * [tmin, D.w]; hits[4i+2] = primIx or ~0. any_hit bit 1: the BVHs with
 * 8-bit quantized child boxes instead of fp32 ones. counts (optional): uint2 per ray = (nodes visited, triangles tested).
 * No context or GPU needed. */
tr_status tr_trace_host(const tr_scene_desc* scene, const float* O4, const float* D4, uint32_t n, float tmin,
                        int32_t any_hit, uint32_t* hits, uint32_t* counts);

#ifdef __cplusplus
}
#endif

#endif /* TRAYRACER_H */

// Device-resident data layout of the wavefront path tracer (shared by the host
// build code and the kernels).
#pragma once

#include "tr_vec.h"
#include "../../include/trayracer.h"

namespace tr {

// Shading record of one triangle: fp32 positions, fp16 texcoords and vertex
// normals, fp16 face normal. Same content and 72-byte layout as the
// reference's PackedTriangle (Tracer/Common/CommonStructs.h:219-253) so the
// shading code reads the same values; fp16 fields are stored as raw bits.
struct alignas(8) TriShade {
    float v0x, v0y, v0z;
    uint16_t uv0x, uv0y, N0x, N0y, N0z, Nx;
    float v1x, v1y, v1z;
    uint16_t uv1x, uv1y, N1x, N1y, N1z, Ny;
    float v2x, v2y, v2z;
    uint16_t uv2x, uv2y, N2x, N2y, N2z, Nz;
};
static_assert(sizeof(TriShade) == 72, "TriShade must stay 72 bytes");

// Resolved constant material. The reference resolves its 13 fp16 properties
// per hit (GetIntersectionAttributes, Tracer/CUDA/GPU/CudaMaterial.h:117-175);
// without textures the resolution is per material, done once on upload with
// the same formulas (emissive = Emissive * diffuse, tint from CIE XYZ,
// luminance = Y).
struct alignas(16) Material {
    float3 diffuse;
    float metallic;
    float3 emissive;
    float subsurface;
    float3 tint;
    float specular;
    float roughness;
    float specularTint;
    float anisotropic;
    float sheen;
    float sheenTint;
    float clearcoat;
    float clearcoatGloss;
    float luminance;
    uint32_t closure;
    uint32_t isEmissive;   // emissive.x + .y + .z > Epsilon (PathTracing.h:73)
    uint32_t texMask;      // bit TR_PROP_* set: that property has a texture (TexSlots)
    uint32_t pad1;
};
static_assert(sizeof(Material) == 96, "Material must stay 96 bytes");

// Textures of one material, read only when its texMask is non-zero: the texture
// object of each property (0 = none) and the fp16-rounded Emissive colour, which
// the per-hit resolution multiplies with the textured diffuse (CudaMaterial.h:158).
struct alignas(16) TexSlots {
    unsigned long long tex[TR_PROP_COUNT];  // cudaTextureObject_t
    float emissive[3];
    uint32_t pad;
};

// Emissive triangle in world space: same fields and 80-byte layout as the
// reference's LightTriangle (Tracer/Common/CommonStructs.h:257-273).
struct alignas(16) LightTri {
    float3 V0;
    int32_t instIx;
    float3 V1;
    int32_t triIx;
    float3 V2;
    float area;
    float3 N;
    float energy;
    float3 radiance;
    float sumEnergy;     // exclusive prefix of energy
};
static_assert(sizeof(LightTri) == 80, "LightTri must stay 80 bytes");

// One entry of the Walker/Vose alias table over the lights.
struct AliasEntry {
    float prob;      // probability of keeping this bucket
    uint32_t alias;  // bucket taken otherwise
};

// 8-wide BVH nodes with the child and leaf encoding of the compressed wide BVH
// (Ylitie, Karras, Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs", HPG 2017), in two layouts.
// meta: 0 empty; internal child = 0x20 | (24 + slot); leaf = (unary triangle
// count << 5) | triangle offset from tri_base. The internal children (the
// node's imask) are the meta bytes whose low five bits are 24 or more.
//
// WideNode, child boxes in fp32, 208 bytes:
//   hdr: child_base, tri_base, meta[0..3], meta[4..7]
//   lo[a][slot], hi[a][slot]: the child boxes per axis (empty slot: +inf / -inf)
// No per-child byte unpacking in the traversal, whose issue slots bound it;
// used while the nodes stay L2-resident (the heightfield's 214k nodes: 45 MB).
struct alignas(16) WideNode {
    uint4 hdr;
    float lo[3][8];
    float hi[3][8];
};
static_assert(sizeof(WideNode) == 208, "WideNode must stay 208 bytes");

// QuantNode, child boxes 8-bit quantized (the paper's layout), 80 bytes:
//   w0: p.x, p.y, p.z (float bits), e.x | e.y<<8 | e.z<<16 | imask<<24
//   w1: child_base, tri_base, meta[0..3], meta[4..7]
//   w2: qlo.x[0..7], qlo.y[0..7]
//   w3: qlo.z[0..7], qhi.x[0..7]
//   w4: qhi.y[0..7], qhi.z[0..7]
// e are biased exponents (scale = 2^(e-127)); a child box is p + q * scale,
// rounded outwards. For BVHs too large for L2.
struct alignas(16) QuantNode {
    uint4 w[5];
};
static_assert(sizeof(QuantNode) == 80, "QuantNode must stay 80 bytes");

// Scene as seen by the kernels (constant for one uploaded scene).
// Preetham sky (CudaSky.h:105-156) with every term that does not depend on the
// ray direction evaluated once on the host (tr_sky.h make_sky).
struct SkyView {
    float3 sunDir;
    uint32_t enabled;
    float3 betaR;          // TotalRayleigh * rayleigh coefficient
    float drawSun;         // 1 or 0
    float3 betaM;          // TotalMie * mie coefficient
    float sunE;            // SunIntensity(cos sun-up angle)
    float3 betaSum;        // betaR + betaM
    float cosSunAngularDiameter;
    float horizonMix;      // saturate((1 - cos sun-up angle)^5)
    float exponent;        // 1 / (1 + sunfade)
    float sunEnergy;       // Sky::SunEnergy (NEE pick weight)
    float sunArea;
};

// Counters of the counting launches (TR_FLAG_COUNT_TRAVERSAL), FrameView::traversal.
constexpr uint32_t kTraversalCounters = 6;

// Default bound on the node visits (internal and leaf groups) of one ray's
// traversal; a ray that runs out sets the frame's device error word.
constexpr uint32_t kMaxTraversalSteps = 1u << 22;

struct SceneView {
    const void* nodes;          // WideNode, or QuantNode when quantNodes
    const float4* bvhTris;      // 3 float4 per triangle in BVH order: (v0, bits(primIx)), (e1, 0), (e2, 0)
    const TriShade* tris;       // by primIx
    const uint32_t* matIdx;     // by primIx
    const Material* materials;
    const LightTri* lights;
    const AliasEntry* alias;
    const float4* invTransforms; // 3 float4 per instance (inverse instance transform rows)
    // two-level scenes (null for one mesh): BVH over the instances, the instance
    // of each of its leaf slots, and per instance (BVH root node, first triangle)
    const void* tlasNodes;      // the same layout as nodes
    const uint32_t* tlasInst;
    const uint2* instInfo;
    int32_t lightCount;
    float lightEnergy;          // reference: last exclusive prefix (Renderer.cpp:500)
    float lightEnergyTotal;     // sum of all light energies
    uint32_t nodeCount;
    uint32_t triCount;
    uint32_t stepLimit = kMaxTraversalSteps;  // bound on node visits of one ray (Settings::stepLimit per launch)
    uint32_t quantNodes = 0;    // nodes and tlasNodes are QuantNode arrays (else WideNode)
    const TexSlots* texSlots;   // per material, null when the scene has no textures
    SkyView sky;
};

struct BatchItem;

// Batched rendering: one continuous wavefront over the samples of many scenes
// whose buffers are concatenated (node, triangle, material and light indices
// rebased). A sample is identified by its sample id: the items' samples are
// numbered item by item, and within an item pixel by pixel with the samples of
// a pixel consecutive (id = item.sampleBase + pixel * spp + sample). A pool of
// path slots is kept full: every iteration traces the paths carried over from
// the last one and starts new samples in the slots that paths left.
struct BatchState {
    uint32_t cursor;       // next sample id to start
    uint32_t end;          // one past the last sample id
    uint32_t queue;        // extend queue length of the current iteration
    uint32_t carried;      // extend queue entries [0, carried) are carried-over paths; the rest start now
    uint32_t freshBase;    // sample id of extend queue entry `carried`
    uint32_t survivors;    // paths the current iteration carries over (shade's extend-queue appends)
    uint32_t hits;         // hit queue length
    uint32_t shadows;      // shadow queue length (written by this iteration's shade)
    uint32_t extendWork;   // work cursors of the persistent extend / connect launches
    uint32_t connectWork;
    uint32_t iterations;   // iterations that traced rays
    uint32_t connectQueue; // shadow rays of the last iteration, traced by this iteration's connect
    unsigned long long extendRays, shadowRays, hitRays;  // totals over the iterations
};

// Per-frame constants of the wavefront (constant between resizes / setting
// changes). Passed by value as a kernel parameter.
struct FrameView {
    float4* state[2];      // 3 planes each, plane stride = capacity: [0] extend queue, [1] hit queue
    uint4* hits;           // by hit-queue slot
    float4* shadow;        // 3 planes, plane stride = capacity
    float4* radiance;      // by path index
    float4* accumulator;   // by pixel
    float4* albedo;        // by pixel (optional)
    float4* normals;       // by pixel (optional)
    float4* colors;        // by pixel
    uint32_t* counters;    // kCounterWords words, layout above
    uint32_t* sampleCount; // device copy of the accumulated sample count
    uint32_t* errorFlag;   // set by bounded loops that ran out
    unsigned long long* traversal;  // kTraversalCounters words (counting launches): extend nodes, extend tris,
                                    // connect nodes, connect tris, shade and connect radiance updates
    uint32_t capacity;
    uint32_t resX, resY;
    uint32_t pathCount;    // resX * resY * multiSample (batched: the pool's path slots)
    // material order of the hit queue (null: shade in queue order)
    const uint32_t* hitOrder;
    // batched rendering only (null / 0 for one scene): the iteration state and
    // the items of the round being rendered (sample ids count from its first item)
    BatchState* batch;
    const BatchItem* items;
    uint32_t itemCount;
    uint32_t pad;
};

struct Camera {
    float3 pos;
    float aperture;
    float3 side;
    float distortion;
    float3 up;
    float focalDist;
    float3 forward;
    float fov;
    int32_t bokehSideCount;
    float bokehRotation;
    float tanFov2;
    float pad;
};

// One scene of a batch: its camera and film, BVH root, light range, pixel
// range in the batch accumulator and sample-id range in its round.
struct BatchItem {
    Camera camera;
    uint32_t width, height;
    uint32_t root;          // BVH root node in the concatenated node array
    uint32_t lightBase;     // first light and alias entry
    int32_t lightCount;
    float lightEnergy;      // last exclusive prefix of the item's lights
    float lightEnergyTotal;
    uint32_t pixelBase;     // first pixel in the batch accumulator
    uint32_t spp;
    uint32_t sampleBase;    // first sample id (counted from the first item of the item's round)
    uint32_t pad1, pad2;
};

// Scratch and parameters of the path-replay adjoint (by path index, plane
// stride = the frame's capacity).
struct AdjointView {
    float4* lrem;          // radiance of the path not yet accounted for
    float4* pending;       // 2 planes: (wo, bits(matIx) or ~0), (wi) of the path's last extend direction
    float4* shadowAdj;     // 2 planes by shadow slot: (wo, bits(matIx)), (wiLight, bits(lightIx))
    uint32_t* visible;     // shadow slots found unoccluded
    const float4* pixelGrad;
    float* grads;          // materialCount x kGradSlots
    float scale;
    uint32_t materialCount;
    uint32_t sampleBase;   // sample count before the replayed frame (its paths' sample keys start here)
    uint32_t pad;
};

// Buffers of the material sort of the hit queue.
struct SortView {
    uint32_t* keys;        // material of each hit-queue slot
    uint32_t* order;       // hit-queue slots grouped by material
    uint32_t* counts;      // hits per material (zeroed again by the scan)
    uint32_t* cursor;      // next free position per material
    uint32_t bins;         // materials
    uint32_t pad;
};

struct Settings {
    uint32_t multiSample;
    uint32_t maxDepth;
    uint32_t seed;
    float rayEpsilon;
    uint32_t rrStart;
    uint32_t flags;
    float maxColor;
    uint32_t refillBelow;  // persistent traversal warps refill lanes below this many active (set per launch)
    uint32_t renderMode;   // RenderModes (Tracer/Common/CommonStructs.h:110-125); 7 = path tracing
    uint32_t renderFlags;  // MaterialPropertyIds for the material-property mode
    float aoDist;          // KernelSettings::aoDist (ambient occlusion modes)
    float zDepthMax;       // KernelSettings::zDepthMax (depth mode)
    uint32_t stepLimit;    // bound on the BVH node visits of one ray (tr_kernel_settings.traversal_step_limit)
};

// RenderModes, Tracer/Common/CommonStructs.h:110-125
constexpr uint32_t kModeAO = 0, kModeAOShading = 1, kModeBitangent = 2, kModeGeometricNormal = 3,
                   kModeMaterialID = 4, kModeMaterialProperty = 5, kModeObjectID = 6, kModePathTracing = 7,
                   kModeShadingNormal = 8, kModeTangent = 9, kModeTextureCoordinate = 10, kModeWireframe = 11,
                   kModeZDepth = 12;

// Device counter words: per bounce the extend queue length, the shadow queue
// length, the work-fetch cursors of the persistent extend and connect launches,
// the hit queue length (rays of the extend queue that hit something), and the
// number of unoccluded shadow rays (adjoint replay only).
constexpr uint32_t kShadowCounterBase = TR_MAX_DEPTH + 1;
constexpr uint32_t kExtendWorkBase = 2 * (TR_MAX_DEPTH + 1);
constexpr uint32_t kConnectWorkBase = 3 * (TR_MAX_DEPTH + 1);
constexpr uint32_t kHitCounterBase = 4 * (TR_MAX_DEPTH + 1);
constexpr uint32_t kVisibleCounterBase = 5 * (TR_MAX_DEPTH + 1);
constexpr uint32_t kCounterWords = 6 * (TR_MAX_DEPTH + 1);

// Path index / flag packing, Tracer/Common/CommonStructs.h:46-71.
constexpr uint32_t kPathIxShift = 4;
constexpr uint32_t kFlagsMask = (1u << kPathIxShift) - 1;
constexpr uint32_t kFlagSpecular = 1u;  // BsdfFlags::Specular, Shade/BSDF/Closure.h:7-11
TR_HD uint32_t pack_path(uint32_t pathIx, uint32_t flags) { return (pathIx << kPathIxShift) | (flags & kFlagsMask); }
TR_HD uint32_t path_ix(uint32_t packed) { return packed >> kPathIxShift; }
TR_HD uint32_t path_flags(uint32_t packed) { return packed & kFlagsMask; }

} // namespace tr

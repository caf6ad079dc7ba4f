/*
 * oracle.h - CPU oracle of the wavefront path-tracing hot path.
 *
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py may load this library, and only as the checker or
 * the timed CPU baseline. The product path (libtrayracer.so) never calls it.
 *
 * A host restatement of the reference's shading and sampling code, templated
 * on the arithmetic type (float: parity with the GPU kernels; double: the FP64
 * image oracle), with its own binary BVH and the same fp32 triangle test the
 * GPU traversal uses. Sources followed (rdbruijne/trayracer):
 *   camera        Tracer/Optix/GPU/optix.cu:51-174
 *   shade         Tracer/CUDA/GPU/Shade/PathTracing.h:8-175
 *   lights        Tracer/CUDA/GPU/CudaLights.h:13-124
 *   attributes    Tracer/CUDA/GPU/CudaMaterial.h:77-212
 *   closures      Tracer/CUDA/GPU/Shade/BSDF/{Closure,Lambert,Diffuse,Disney,Microfacet}.h
 *   utilities     Tracer/CUDA/GPU/CudaUtility.h, CudaLinearMath.h
 *   RNG           thirdparty/CUDA/random.h:31-67
 *   flattening    Tracer/Resources/Model.cpp:93-236, Tracer/Renderer/Scene.cpp:275-302,
 *                 Tracer/Resources/Material.cpp:56-78
 *   frame loop    Tracer/Renderer/DeviceRenderer.cpp:97-274
 * Buffers use the same layouts as the C ABI (include/trayracer.h).
 */
#ifndef TRAYRACER_ORACLE_H
#define TRAYRACER_ORACLE_H

#include <stdint.h>

#include "../include/trayracer.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene orc_scene;

orc_scene* orc_scene_create(const tr_scene_desc* desc);
void orc_scene_destroy(orc_scene* s);
uint32_t orc_light_count(const orc_scene* s);
/* total = 0: the reference's LightEnergy (last exclusive prefix); 1: sum. */
float orc_light_energy(const orc_scene* s, int total);

/* Camera rays of paths [first, first + n) of one frame: writes float4 planes
 * (O, bits(pathIx << 4)), (D, 0), (T, T, T, 1), each n entries. */
void orc_generate(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t width,
                  uint32_t height, uint32_t sample_count, uint32_t first, uint32_t n, float* O4, float* D4,
                  float* T4);

/* Closest hit of n rays (float4 O, float4 D) over [tmin, 1e30]; writes uint4
 * (bary 16:16, instIx, primIx, bits(t)), miss = (0, ~0, ~0, bits(1e30)). */
void orc_trace_closest(const orc_scene* s, const float* O4, const float* D4, uint32_t n, float tmin,
                       uint32_t* hits);

/* One ray over [tmin, tmax]: closest hit (any = 0) or first hit (any = 1).
 * Returns 1 on a hit with prim, t and barycentrics (u, v) set. */
// tex2D<float4> of texture `texture` at (u, v) as the device samples it (bilinear,
// wrap, normalised coordinates, 8-bit fractional weights).
void orc_texture_sample(const orc_scene* s, uint32_t texture, float u, float v, float* out);
// Sky seen by paths that leave the scene (NULL: disabled, the default).
void orc_set_sky(orc_scene* s, const tr_sky_desc* sky);
// RayPickResult (9 words) of the RayPick raygen for pixel (x, y).
void orc_pick_ray(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t width,
                  uint32_t height, int32_t x, int32_t y, float* out);
int orc_trace_ray(const orc_scene* s, const float* O, const float* D, float tmin, float tmax, int any, uint32_t* prim,
                  float* t, float* u, float* v, uint32_t* inst);

/* All triangles whose hit distance lies within rel_tol of t (near ties of a
 * closest hit). Writes up to max_out primitive indices, returns the count. */
uint32_t orc_ties(const orc_scene* s, const float* O, const float* D, float tmin, float t, float rel_tol,
                  uint32_t* prims, uint32_t max_out, uint32_t* insts);

/* Shadow rays (float4 O, float4 (L, dist)): occluded[i] = any hit in
 * [eps, dist - 2 eps]. */
void orc_trace_any(const orc_scene* s, const float* O4, const float* L4, uint32_t n, float eps, uint8_t* occluded);

/* Shades n queue entries (float4 planes O4, D4, T4 and uint4 hits). Outputs are
 * per input entry (not compacted): ext (3 float4 planes), ext_valid, shadow
 * (3 float4 planes), sh_valid, and the radiance added by the shade stage. */
void orc_shade(const orc_scene* s, const tr_kernel_settings* st, uint32_t bounce, uint32_t sample_count,
               uint32_t width, uint32_t height, uint32_t n, const float* O4, const float* D4, const float* T4,
               const uint32_t* hits, float* ext, uint8_t* ext_valid, float* sh, uint8_t* sh_valid,
               float* radiance_add);

/* orc_shade computed in double (outputs rounded to float): the conditioning
 * reference for comparisons of fp32 shading. */
void orc_shade_fp64(const orc_scene* s, const tr_kernel_settings* st, uint32_t bounce, uint32_t sample_count,
                    uint32_t width, uint32_t height, uint32_t n, const float* O4, const float* D4, const float* T4,
                    const uint32_t* hits, float* ext, uint8_t* ext_valid, float* sh, uint8_t* sh_valid,
                    float* radiance_add);

/* Renders `frames` frames of multi_sample samples for pixels
 * [first_pixel, first_pixel + pixel_count), each path traced depth first with
 * the same per-path random streams as the wavefront. Writes per path the
 * radiance of the last frame (path_radiance, 4 doubles per path index of the
 * selected pixels x multi_sample, may be NULL) and per pixel the accumulator
 * (4 doubles: rgb sum over all frames, sample count). use_double selects the
 * FP64 instantiation. ray_counts[0..1] += extend rays, shadow rays. Returns 0. */
int orc_render(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t width,
               uint32_t height, uint32_t frames, uint32_t first_pixel, uint32_t pixel_count, int use_double,
               int threads, double* accumulator, double* path_radiance, uint64_t* ray_counts);

/* One closure on explicit inputs (tr_closure type; reference = 1 keeps the
 * reference's Disney behaviour). in (31 floats): wo[3], wi[3], T[3], the
 * HitMaterial fields in declaration order (CudaMaterial.h:31-52: diffuse[3],
 * metallic, emissive[3], subsurface, tint[3], specular, roughness,
 * specularTint, anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss,
 * luminance), r0, r1. out (14 floats): extend T[3], pdf, wi[3], bits(flags),
 * shadow T[3], pdf, 0, 0. */
void orc_closure(int type, int reference, int use_double, const float* in, float* out);

/* Path-replay gradient (default sampling mode) of the frame with the given
 * sample_count: adds to grads (material_count x 9 doubles: base colour rgb,
 * roughness, metallic, specular, emission rgb) the gradient of a loss whose
 * derivative with respect to each path's radiance is scale * pixel_grad[pixel]
 * (float4 per pixel). use_double selects the FP64 instantiation. Returns 0,
 * or 1 for the reference sampling mode (not differentiated). */
int orc_adjoint(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t width,
                uint32_t height, uint32_t sample_count, const float* pixel_grad, float scale, int use_double,
                int threads, double* grads);

/* Closure value of a scene material at tangent-space (wo, wi) in the default
 * mode with its derivatives: out[7c] = f_c, out[7c+1+p] = d f_c / d param p
 * (base colour rgb, roughness, metallic, specular), c = 0..2. */
void orc_closure_value_grad(const orc_scene* s, uint32_t material, const float* wo, const float* wi, double* out);

/* Random numbers of the counter-based stream (testing): the first n draws
 * of (pixel, sample, bounce, seed). */
void orc_counter_rng(uint32_t pixel, uint32_t sample, uint32_t bounce, uint32_t seed, uint32_t n, float* out);
/* Order of the random draws the reference takes as arguments of one call
 * (optix.cu:55,147, CudaLights.h:107, PathTracing.h:129), which C++ leaves
 * unspecified: 0 = left to right (the GPU kernels), 1 = right to left (the
 * g++ host build of the reference in oracle/_ref). Reference sampling only. */
void orc_set_reference_draw_order(int right_to_left);

/* Random numbers of the reference stream: tea<2>(v0, v1) then n LCG draws. */
void orc_reference_rng(uint32_t v0, uint32_t v1, uint32_t n, float* out);

#ifdef __cplusplus
}
#endif

#endif

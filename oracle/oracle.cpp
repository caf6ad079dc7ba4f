// CPU oracle of the wavefront path-tracing hot path (test infrastructure).
//
// Restates the reference's shading/sampling code (file:line in each function)
// templated on the arithmetic type T: T = float checks the GPU kernels,
// T = double is the FP64 image oracle. Compiled with -ffp-contract=off so
// every float operation rounds where the source says it does.
#include "oracle.h"

#include <cuda_fp16.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

// ------------------------------------------------------------------ scalars
// Math entry points for float, double and the dual numbers of the adjoint.
template <class T> inline T msqrt(T x) { using std::sqrt; return sqrt(x); }
template <class T> inline T mfabs(T x) { using std::fabs; return fabs(x); }
template <class T> inline T mlog(T x) { using std::log; return log(x); }

// Forward-mode dual number over B (double for the FP64 gradient): value and
// derivatives with respect to base colour r, g, b, roughness, metallic, specular.
constexpr int kDP = 6;
template <class B>
struct DualT {
    B v;
    B d[kDP];
    DualT() : v(0) { for (int i = 0; i < kDP; ++i) d[i] = 0; }
    DualT(double x) : v(B(x)) { for (int i = 0; i < kDP; ++i) d[i] = 0; }
    static DualT var(B x, int k) { DualT r(0.0); r.v = x; r.d[k] = 1; return r; }
};
template <class B> inline DualT<B> operator+(const DualT<B>& a, const DualT<B>& b)
{ DualT<B> r; r.v = a.v + b.v; for (int i = 0; i < kDP; ++i) r.d[i] = a.d[i] + b.d[i]; return r; }
template <class B> inline DualT<B> operator-(const DualT<B>& a, const DualT<B>& b)
{ DualT<B> r; r.v = a.v - b.v; for (int i = 0; i < kDP; ++i) r.d[i] = a.d[i] - b.d[i]; return r; }
template <class B> inline DualT<B> operator-(const DualT<B>& a)
{ DualT<B> r; r.v = -a.v; for (int i = 0; i < kDP; ++i) r.d[i] = -a.d[i]; return r; }
template <class B> inline DualT<B> operator*(const DualT<B>& a, const DualT<B>& b)
{ DualT<B> r; r.v = a.v * b.v; for (int i = 0; i < kDP; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i]; return r; }
template <class B> inline DualT<B> operator/(const DualT<B>& a, const DualT<B>& b)
{ DualT<B> r; r.v = a.v / b.v; for (int i = 0; i < kDP; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) / b.v; return r; }
template <class B> inline DualT<B> sqrt(const DualT<B>& a)
{ DualT<B> r; r.v = std::sqrt(a.v); const B k = r.v > 0 ? B(0.5) / r.v : B(0); for (int i = 0; i < kDP; ++i) r.d[i] = a.d[i] * k; return r; }
template <class B> inline DualT<B> fabs(const DualT<B>& a) { return a.v < 0 ? -a : a; }
template <class B> inline DualT<B> log(const DualT<B>& a)
{ DualT<B> r; r.v = std::log(a.v); for (int i = 0; i < kDP; ++i) r.d[i] = a.d[i] / a.v; return r; }
template <class B> inline bool operator<(const DualT<B>& a, const DualT<B>& b) { return a.v < b.v; }
template <class B> inline bool operator>(const DualT<B>& a, const DualT<B>& b) { return a.v > b.v; }
template <class B> inline bool operator<=(const DualT<B>& a, const DualT<B>& b) { return a.v <= b.v; }
template <class B> inline bool operator==(const DualT<B>& a, const DualT<B>& b) { return a.v == b.v; }
template <class B> inline bool operator!=(const DualT<B>& a, const DualT<B>& b) { return a.v != b.v; }
template <class B> inline bool operator<(const DualT<B>& a, double b) { return a.v < b; }
template <class B> inline bool operator>(const DualT<B>& a, double b) { return a.v > b; }
template <class B> inline bool operator==(const DualT<B>& a, double b) { return a.v == b; }
template <class B> inline bool operator!=(const DualT<B>& a, double b) { return a.v != b; }
template <class B> inline bool operator<(const DualT<B>& a, int b) { return a.v < b; }
template <class B> inline bool operator>(const DualT<B>& a, int b) { return a.v > b; }
template <class B> inline bool operator<=(const DualT<B>& a, int b) { return a.v <= b; }
template <class B> inline DualT<B> operator+(const DualT<B>& a, double b) { return a + DualT<B>(b); }
template <class B> inline DualT<B> operator+(double b, const DualT<B>& a) { return DualT<B>(b) + a; }
template <class B> inline DualT<B> operator-(const DualT<B>& a, double b) { return a - DualT<B>(b); }
template <class B> inline DualT<B> operator-(double b, const DualT<B>& a) { return DualT<B>(b) - a; }
template <class B> inline DualT<B> operator*(const DualT<B>& a, double b) { return a * DualT<B>(b); }
template <class B> inline DualT<B> operator*(double b, const DualT<B>& a) { return DualT<B>(b) * a; }
template <class B> inline DualT<B> operator/(const DualT<B>& a, double b) { return a / DualT<B>(b); }
template <class B> inline DualT<B> operator/(double b, const DualT<B>& a) { return DualT<B>(b) / a; }

// ------------------------------------------------------------------ vectors
template <class T>
struct V3 {
    T x, y, z;
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> v3s(T s) { return V3<T>{s, s, s}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> inline V3<T> operator+(T s, V3<T> a) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T length(V3<T> v) { return msqrt(dot(v, v)); }
// helper_math normalize: v * rsqrtf(dot(v, v)); host rsqrtf = 1 / sqrtf
template <class T> inline V3<T> normalize(V3<T> v) { return v * (T(1) / msqrt(dot(v, v))); }
template <class T> inline T sq(T x) { return x * x; }
template <class T> inline T mix(T a, T b, T t) { return (a * (T(1) - t)) + (b * t); }
template <class T> inline T lerp(T a, T b, T t) { return a + t * (b - a); }
template <class T> inline T fmx(T a, T b) { return a > b ? a : b; }   // fmaxf, non-NaN inputs
template <class T> inline T fmn(T a, T b) { return a < b ? a : b; }
template <class T> inline T clampT(T x, T lo, T hi) { return fmx(lo, fmn(x, hi)); }
template <class T> inline T saturate(T x) { return x < T(0) ? T(0) : (x > T(1) ? T(1) : x); }
template <class T> inline V3<T> reflect(V3<T> i, V3<T> n) { return i - T(2) * n * dot(n, i); }
template <class T> inline bool finite3(V3<T> c) { return std::isfinite(c.x + c.y + c.z); }

template <class T> struct K {
    static constexpr T Pi = T(3.1415926535897932);
    static constexpr T TwoPi = T(6.2831853071795865);
    static constexpr T RcpPi = T(0.3183098861837907);
    static constexpr T RcpTwoPi = T(0.1591549430918953);
    static constexpr T PiOver2 = T(1.57079632679);
    static constexpr T PiOver4 = T(0.78539816339);
};
template <> struct K<float> {
    static constexpr float Pi = 3.1415926535897932f;
    static constexpr float TwoPi = 6.2831853071795865f;
    static constexpr float RcpPi = 0.3183098861837907f;
    static constexpr float RcpTwoPi = 0.1591549430918953f;
    static constexpr float PiOver2 = 1.57079632679f;
    static constexpr float PiOver4 = 0.78539816339f;
};
template <class B> struct K<DualT<B>> {
    static inline const DualT<B> Pi = DualT<B>(3.1415926535897932);
    static inline const DualT<B> TwoPi = DualT<B>(6.2831853071795865);
    static inline const DualT<B> RcpPi = DualT<B>(0.3183098861837907);
    static inline const DualT<B> RcpTwoPi = DualT<B>(0.1591549430918953);
    static inline const DualT<B> PiOver2 = DualT<B>(1.57079632679);
    static inline const DualT<B> PiOver4 = DualT<B>(0.78539816339);
};
constexpr float kEps = 1e-3f;   // CudaGlobals.h:10
constexpr float kDstMax = 1e30f; // optix.cu:16

inline uint32_t f2u(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

inline uint16_t hbits(float x)
{
    const __half h = __float2half(x);
    const __half_raw r = h;
    return r.x;
}
inline float hval(uint16_t b)
{
    __half_raw r;
    r.x = b;
    return __half2float(__half(r));
}
inline float hround(float x) { return hval(hbits(x)); }

// ------------------------------------------------------------------ RNG
// thirdparty/CUDA/random.h:31-67
inline uint32_t tea2(uint32_t v0, uint32_t v1)
{
    uint32_t s0 = 0;
    for (int n = 0; n < 2; ++n) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
struct RefRng {
    uint32_t state;
    float next()
    {
        state = 1664525u * state + 1013904223u;
        return float(state & 0x00FFFFFFu) / float(0x01000000);
    }
};
// pcg4d, Jarzynski & Olano, JCGT 9(3) 2020
inline void pcg4d(uint32_t v[4])
{
    for (int i = 0; i < 4; ++i)
        v[i] = v[i] * 1664525u + 1013904223u;
    v[0] += v[1] * v[3];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
    v[3] += v[1] * v[2];
    for (int i = 0; i < 4; ++i)
        v[i] ^= v[i] >> 16;
    v[0] += v[1] * v[3];
    v[1] += v[2] * v[0];
    v[2] += v[0] * v[1];
    v[3] += v[1] * v[2];
}
struct CounterRng {
    uint32_t pixel, sample, bounce, seed, dim = 0;
    uint32_t block[4];
    float next()
    {
        if ((dim & 3u) == 0) {
            block[0] = pixel;
            block[1] = sample;
            block[2] = (bounce << 8) | (dim >> 2);
            block[3] = seed;
            pcg4d(block);
        }
        const uint32_t w = block[dim & 3u];
        ++dim;
        return float(w >> 8) * (1.0f / 16777216.0f);
    }
};

// ------------------------------------------------------------------ scene
struct Tri {
    float v[3][3];
    uint16_t uv[3][2];
    uint16_t n[3][3];
    uint16_t N[3];
};
struct MatRaw {            // fp16-rounded properties (Material::Property::Build)
    float diffuse[3];
    float emissive[3];
    float metallic, subsurface, specular, roughness, specularTint, anisotropic, sheen, sheenTint, clearcoat,
        clearcoatGloss;
    uint32_t closure;
};
struct Texture {            // RGBA binary16 texels, row by row
    uint32_t w = 0, h = 0;
    std::vector<uint16_t> texels;
};
struct Light {
    float V0[3], V1[3], V2[3], N[3];
    float area, energy, radiance[3], sumEnergy;
    uint32_t triIx;
};
struct Alias {
    float prob;
    uint32_t alias;
};
struct Node {
    float lo[3], hi[3];
    uint32_t first;   // internal: left child (right = left + 1); leaf: first ref
    uint32_t count;   // 0 = internal
};

} // namespace

struct orc_scene {
    std::vector<Tri> tris;
    std::vector<float> geo;      // 9 floats per triangle: v0, e1 = v1 - v0, e2 = v2 - v0 (float rounding)
    std::vector<double> geoD;    // 9 doubles per triangle: v0, e1, e2 (exact)
    std::vector<uint32_t> matIdx;
    std::vector<MatRaw> mats;
    std::vector<Texture> textures;
    std::vector<int32_t> matTex;   // TR_PROP_COUNT texture indices per material (-1: none); empty: no textures
    std::vector<Light> lights;
    std::vector<Alias> alias;
    float lightEnergy = 0.f;
    float lightEnergyTotal = 0.f;
    std::vector<Node> nodes;
    std::vector<uint32_t> refs;
    // two-level scenes: meshes placed by instances, one BVH per mesh (refs are
    // global triangle indices), the inverse transform rows (r | t) per instance
    bool twoLevel = false;
    std::vector<uint32_t> meshTriBase, meshTriCount, instMesh;
    std::vector<float> instInv;
    std::vector<std::vector<Node>> meshNodes;
    std::vector<std::vector<uint32_t>> meshRefs;
    // Sky::Build (Sky.cpp): the SkyData fields SampleSky reads; disabled by default
    struct {
        float sunDir[3] = {0.f, 1.f, 0.f};
        int enabled = 0;
        float drawSun = 0.f;
        float cosSunAngularDiameter = 1.f;
        float sunIntensity = 0.f;
        float turbidity = 4.f;
    } sky;
};

namespace {

// Walker/Vose alias table: small/large lists in index order, consumed from the back.
std::vector<Alias> alias_table(const std::vector<double>& w)
{
    const size_t n = w.size();
    std::vector<Alias> t(n);
    if (!n)
        return t;
    double total = 0;
    for (double x : w)
        total += x;
    std::vector<double> sc(n);
    std::vector<uint32_t> small, large;
    for (size_t i = 0; i < n; ++i) {
        sc[i] = total > 0 ? w[i] * double(n) / total : 1.0;
        (sc[i] < 1.0 ? small : large).push_back(uint32_t(i));
    }
    while (!small.empty() && !large.empty()) {
        const uint32_t s = small.back();
        small.pop_back();
        const uint32_t l = large.back();
        large.pop_back();
        t[s].prob = float(sc[s]);
        t[s].alias = l;
        sc[l] = (sc[l] + sc[s]) - 1.0;
        (sc[l] < 1.0 ? small : large).push_back(l);
    }
    for (uint32_t l : large) t[l] = Alias{1.f, l};
    for (uint32_t s : small) t[s] = Alias{1.f, s};
    return t;
}

// Median-split BVH over the triangles [base, base + n) (refs hold global indices).
void build_bvh_range(const orc_scene& S, uint32_t base, uint32_t n, std::vector<Node>& nodes,
                     std::vector<uint32_t>& refs)
{
    refs.resize(n);
    for (uint32_t i = 0; i < n; ++i)
        refs[i] = base + i;
    nodes.clear();
    nodes.reserve(2 * size_t(n) + 1);
    std::vector<float> c(3 * size_t(S.tris.size()));
    for (uint32_t i = base; i < base + n; ++i)
        for (int a = 0; a < 3; ++a)
            c[3 * size_t(i) + a] = (S.tris[i].v[0][a] + S.tris[i].v[1][a] + S.tris[i].v[2][a]) / 3.f;
    struct Item {
        uint32_t node, begin, end;
    };
    nodes.push_back(Node{});
    std::vector<Item> stack{{0, 0, n}};
    while (!stack.empty()) {
        const Item it = stack.back();
        stack.pop_back();
        Node nd{};
        for (int a = 0; a < 3; ++a) {
            nd.lo[a] = INFINITY;
            nd.hi[a] = -INFINITY;
        }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t k = it.begin; k < it.end; ++k) {
            const Tri& t = S.tris[refs[k]];
            for (int v = 0; v < 3; ++v)
                for (int a = 0; a < 3; ++a) {
                    nd.lo[a] = std::min(nd.lo[a], t.v[v][a]);
                    nd.hi[a] = std::max(nd.hi[a], t.v[v][a]);
                }
            for (int a = 0; a < 3; ++a) {
                clo[a] = std::min(clo[a], c[3 * refs[k] + a]);
                chi[a] = std::max(chi[a], c[3 * refs[k] + a]);
            }
        }
        const uint32_t cnt = it.end - it.begin;
        if (cnt <= 4) {
            nd.first = it.begin;
            nd.count = cnt;
            nodes[it.node] = nd;
            continue;
        }
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis])
                axis = a;
        const uint32_t mid = it.begin + cnt / 2;
        std::nth_element(refs.begin() + it.begin, refs.begin() + mid, refs.begin() + it.end,
                         [&](uint32_t x, uint32_t y) { return c[3 * x + axis] < c[3 * y + axis]; });
        const uint32_t left = uint32_t(nodes.size());
        nodes.push_back(Node{});
        nodes.push_back(Node{});
        nd.first = left;
        nd.count = 0;
        nodes[it.node] = nd;
        stack.push_back({left, it.begin, mid});
        stack.push_back({left + 1, mid, it.end});
    }
}

void build_bvh(orc_scene& S)
{
    if (!S.twoLevel) {
        build_bvh_range(S, 0, uint32_t(S.tris.size()), S.nodes, S.refs);
        return;
    }
    S.meshNodes.resize(S.meshTriBase.size());
    S.meshRefs.resize(S.meshTriBase.size());
    for (size_t m = 0; m < S.meshTriBase.size(); ++m)
        build_bvh_range(S, S.meshTriBase[m], S.meshTriCount[m], S.meshNodes[m], S.meshRefs[m]);
}

// ---------------------------------------------------------------- triangle test
// Moller-Trumbore on (v0, e1, e2), the same operation sequence as the GPU
// traversal (explicit fused multiply-adds, round-to-nearest products).
inline bool tri_test_f(const float* g, const float O[3], const float D[3], float tmin, float tmax, float& t,
                       float& u, float& v)
{
    const float* a = g;
    const float* b = g + 3;
    const float* c = g + 6;
    const float px = std::fma(D[1], c[2], -(D[2] * c[1]));
    const float py = std::fma(D[2], c[0], -(D[0] * c[2]));
    const float pz = std::fma(D[0], c[1], -(D[1] * c[0]));
    const float det = std::fma(b[0], px, std::fma(b[1], py, b[2] * pz));
    if (det == 0.0f)
        return false;
    const float inv = 1.0f / det;
    const float tx = O[0] - a[0], ty = O[1] - a[1], tz = O[2] - a[2];
    const float uu = std::fma(tx, px, std::fma(ty, py, tz * pz)) * inv;
    if (!(uu >= 0.0f && uu <= 1.0f))
        return false;
    const float qx = std::fma(ty, b[2], -(tz * b[1]));
    const float qy = std::fma(tz, b[0], -(tx * b[2]));
    const float qz = std::fma(tx, b[1], -(ty * b[0]));
    const float vv = std::fma(D[0], qx, std::fma(D[1], qy, D[2] * qz)) * inv;
    if (!(vv >= 0.0f && uu + vv <= 1.0f))
        return false;
    const float tt = std::fma(c[0], qx, std::fma(c[1], qy, c[2] * qz)) * inv;
    if (!(tt >= tmin && tt <= tmax))
        return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

inline bool tri_test_d(const double* g, const double O[3], const double D[3], double tmin, double tmax, double& t,
                       double& u, double& v)
{
    const double* a = g;
    const double* b = g + 3;
    const double* c = g + 6;
    const double px = D[1] * c[2] - D[2] * c[1];
    const double py = D[2] * c[0] - D[0] * c[2];
    const double pz = D[0] * c[1] - D[1] * c[0];
    const double det = b[0] * px + b[1] * py + b[2] * pz;
    if (det == 0.0)
        return false;
    const double inv = 1.0 / det;
    const double tx = O[0] - a[0], ty = O[1] - a[1], tz = O[2] - a[2];
    const double uu = (tx * px + ty * py + tz * pz) * inv;
    if (!(uu >= 0.0 && uu <= 1.0))
        return false;
    const double qx = ty * b[2] - tz * b[1];
    const double qy = tz * b[0] - tx * b[2];
    const double qz = tx * b[1] - ty * b[0];
    const double vv = (D[0] * qx + D[1] * qy + D[2] * qz) * inv;
    if (!(vv >= 0.0 && uu + vv <= 1.0))
        return false;
    const double tt = (c[0] * qx + c[1] * qy + c[2] * qz) * inv;
    if (!(tt >= tmin && tt <= tmax))
        return false;
    t = tt;
    u = uu;
    v = vv;
    return true;
}

inline bool box_hit(const Node& n, const double O[3], const double inv[3], double tmin, double tmax, double& tnear)
{
    double t0 = tmin, t1 = tmax;
    for (int a = 0; a < 3; ++a) {
        double lo = (double(n.lo[a]) - O[a]) * inv[a];
        double hi = (double(n.hi[a]) - O[a]) * inv[a];
        if (lo > hi)
            std::swap(lo, hi);
        if (std::isnan(lo)) lo = -INFINITY;
        if (std::isnan(hi)) hi = INFINITY;
        t0 = std::max(t0, lo);
        t1 = std::min(t1, hi);
    }
    tnear = t0;
    // slack so that round-off never culls a triangle lying on the box face
    return t0 <= t1 + 1e-9 * std::max(1.0, mfabs(t1));
}

// Closest hit (any = false) or first hit (any = true) of one ray in one BVH; T
// selects the triangle test precision.
template <class T>
bool trace_bvh(const orc_scene& S, const std::vector<Node>& nodes, const std::vector<uint32_t>& refs,
               const T Oin[3], const T Din[3], T tmin, T& tmax, bool any, uint32_t& prim, T& bu, T& bv)
{
    if (nodes.empty() || refs.empty())
        return false;
    double O[3], inv[3];
    for (int a = 0; a < 3; ++a) {
        O[a] = double(Oin[a]);
        inv[a] = 1.0 / double(Din[a]);
    }
    bool found = false;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& n = nodes[stack[--sp]];
        double tn;
        if (!box_hit(n, O, inv, double(tmin), double(tmax), tn))
            continue;
        if (n.count == 0) {
            double tl, tr;
            const bool hl = box_hit(nodes[n.first], O, inv, double(tmin), double(tmax), tl);
            const bool hr = box_hit(nodes[n.first + 1], O, inv, double(tmin), double(tmax), tr);
            if (hl && hr) {
                if (tl <= tr) {
                    stack[sp++] = n.first + 1;
                    stack[sp++] = n.first;
                } else {
                    stack[sp++] = n.first;
                    stack[sp++] = n.first + 1;
                }
            } else if (hl) {
                stack[sp++] = n.first;
            } else if (hr) {
                stack[sp++] = n.first + 1;
            }
            if (sp > 120)
                return found;  // cannot happen for a median-split tree of < 2^60 leaves
            continue;
        }
        for (uint32_t k = n.first; k < n.first + n.count; ++k) {
            const uint32_t p = refs[k];
            T t, u, v;
            bool h;
            if constexpr (sizeof(T) == 4)
                h = tri_test_f(&S.geo[9 * size_t(p)], Oin, Din, tmin, tmax, t, u, v);
            else
                h = tri_test_d(&S.geoD[9 * size_t(p)], Oin, Din, tmin, tmax, t, u, v);
            if (!h)
                continue;
            if (any) {
                tmax = t;
                prim = p;
                return true;
            }
            if (!found || t < tmax || (t == tmax && p < prim)) {
                found = true;
                tmax = t;
                prim = p;
                bu = u;
                bv = v;
            }
        }
    }
    return found;
}

// World ray -> object ray of an instance: rows (r | t) of its inverse transform,
// ((r.x p.x + r.y p.y) + r.z p.z) + t, every operation rounded on its own as the
// GPU traversal does (tr_traverse.cuh xform_point / xform_vector).
template <class T>
void to_object(const float* m, const T O[3], const T D[3], T Oo[3], T Do[3])
{
    for (int r = 0; r < 3; ++r) {
        const T a = T(m[4 * r]), b = T(m[4 * r + 1]), c = T(m[4 * r + 2]), t = T(m[4 * r + 3]);
        Oo[r] = ((a * O[0] + b * O[1]) + c * O[2]) + t;
        Do[r] = (a * D[0] + b * D[1]) + c * D[2];
    }
}

// Closest or first hit of one ray in the scene: one level, or every instance's
// mesh in object space (the ray parameter t is shared; on equal t the earlier
// instance keeps the hit). inst = instance of the hit; prim = global triangle.
template <class T>
bool trace(const orc_scene& S, const T Oin[3], const T Din[3], T tmin, T& tmax, bool any, uint32_t& prim, T& bu,
           T& bv, uint32_t* inst = nullptr)
{
    if (!S.twoLevel) {
        if (inst)
            *inst = 0;
        return trace_bvh<T>(S, S.nodes, S.refs, Oin, Din, tmin, tmax, any, prim, bu, bv);
    }
    bool found = false;
    for (uint32_t i = 0; i < S.instMesh.size(); ++i) {
        T Oo[3], Do[3];
        to_object<T>(&S.instInv[12 * size_t(i)], Oin, Din, Oo, Do);
        const uint32_t m = S.instMesh[i];
        T tm = tmax, u = 0, v = 0;
        uint32_t p = 0;
        if (!trace_bvh<T>(S, S.meshNodes[m], S.meshRefs[m], Oo, Do, tmin, tm, any, p, u, v))
            continue;
        if (any || !found || tm < tmax) {
            found = true;
            tmax = tm;
            prim = p;
            bu = u;
            bv = v;
            if (inst)
                *inst = i;
            if (any)
                return true;
        }
    }
    return found;
}

// ---------------------------------------------------------------- shading types
template <class T>
struct HitMat {
    V3<T> diffuse;
    T metallic;
    V3<T> emissive;
    T subsurface;
    V3<T> tint;
    T specular, roughness, specularTint, anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss, luminance;
    uint32_t closure;
};
template <class T>
struct Lobe {
    V3<T> wi;
    T pdf;
    V3<T> Tv;
    uint32_t flags;
};
template <class T>
struct Clos {
    V3<T> extT;
    T extPdf;
    V3<T> extWi;
    uint32_t extFlags;
    V3<T> shT;
    T shPdf;
};
constexpr uint32_t kSpec = 1u;

// Four reference call sites draw two or three random numbers as arguments of
// one call (optix.cu:55 and :147, CudaLights.h:107, PathTracing.h:129). C++
// leaves the order of those draws unspecified: the oracle draws them left to
// right (as the GPU kernels do) unless g_refRightToLeft is set, which
// reproduces the host (g++) build of the reference in oracle/_ref.
bool g_refRightToLeft = false;

template <class Rng> inline void draw2(Rng& rng, bool rtl, float& a, float& b)
{
    if (rtl) {
        b = rng.next();
        a = rng.next();
    } else {
        a = rng.next();
        b = rng.next();
    }
}
template <class Rng> inline void draw3(Rng& rng, bool rtl, float& a, float& b, float& c)
{
    if (rtl) {
        c = rng.next();
        b = rng.next();
        a = rng.next();
    } else {
        a = rng.next();
        b = rng.next();
        c = rng.next();
    }
}
template <class Rng> constexpr bool is_ref_rng() { return std::is_same<Rng, RefRng>::value; }

template <class T> inline void sincosT(T x, T& s, T& c)
{
    s = std::sin(x);
    c = std::cos(x);
}

// SampleCosineHemisphere, CudaUtility.h:270-280
template <class T> V3<T> cos_hemi(T r0, T r1)
{
    T s, c;
    sincosT(K<T>::TwoPi * r0, s, c);
    const T b = msqrt(T(1) - r1);
    return v3(c * b, s * b, msqrt(r1));
}

// FinalizeClosure, Closure.h:57-74
template <class T> Clos<T> finalize(V3<T> Tp, const Lobe<T>& e, const Lobe<T>& s)
{
    Clos<T> c;
    c.shT = e.Tv * mfabs(e.wi.z) * Tp;
    c.shPdf = e.pdf;
    c.extT = s.Tv * mfabs(s.wi.z) * Tp;
    c.extPdf = s.pdf;
    c.extWi = s.wi;
    c.extFlags = s.flags;
    return c;
}

// LambertClosure, Lambert.h:8-59
template <class T> Clos<T> lambert(V3<T> wo, V3<T> wi, V3<T> Tp, const HitMat<T>& m, T r0, T r1)
{
    Lobe<T> e;
    const T p = m.roughness < T(kEps) ? T(0) : K<T>::RcpPi;
    e.wi = wi;
    e.pdf = p * wi.z;
    e.Tv = v3s(p);
    e.flags = 0;
    Lobe<T> s;
    const T specProb = T(1) - m.roughness;
    if (r0 < specProb) {
        s.wi = reflect(-wo, v3(T(0), T(0), T(1)));
        s.pdf = 1;
        s.Tv = v3s(T(1) / s.wi.z) * m.diffuse;
        s.flags = kSpec;
    } else {
        s.wi = cos_hemi((specProb - r0) / (T(1) - specProb), r1);
        s.pdf = K<T>::RcpPi * s.wi.z;
        s.Tv = v3s(K<T>::RcpPi) * m.diffuse;
        s.flags = 0;
    }
    return finalize(Tp, e, s);
}

// DiffuseClosure, Diffuse.h:8-42
template <class T> Clos<T> diffuse(V3<T> wo, V3<T> wi, V3<T> Tp, const HitMat<T>& m, T r0, T r1)
{
    (void)wo;
    Lobe<T> e{wi, K<T>::RcpPi * wi.z, v3s(K<T>::RcpPi) * m.diffuse, 0};
    const V3<T> w = cos_hemi(r0, r1);
    Lobe<T> s{w, K<T>::RcpPi * w.z, v3s(K<T>::RcpPi) * m.diffuse, 0};
    return finalize(Tp, e, s);
}

// Microfacet.h:33-324
template <class T> void alpha_xy(T rough, T aniso, T& ax, T& ay)
{
    const T r2 = sq(rough);
    const T aspect = msqrt(T(1) + aniso * (aniso < 0 ? T(0.9f) : T(-0.9f)));
    ax = fmx(T(0.001f), r2 / aspect);
    ay = fmx(T(0.001f), r2 * aspect);
}
template <class T> T stretched(V3<T> m, T s, T ax, T ay)
{
    if (ax == ay || s == T(0))
        return T(1) / sq(ax);
    return sq(m.x / (s * ax)) + sq(m.z / (s * ay));
}
template <class T> T projected(V3<T> m, T s, T ax, T ay)
{
    if (ax == ay || s == T(0))
        return ax;
    return msqrt(sq((m.x * ax) / s) + sq((m.y * ay) / s));
}
template <class T> T ggx_lambda(V3<T> v, T ax, T ay)
{
    const T c = v.z;
    if (c == T(0))
        return 0;
    const T c2 = sq(c);
    const T s = msqrt(fmx(T(0), T(1) - c2));
    const T a = projected(v, s, ax, ay);
    const T t2 = sq(s) / c2;
    return (T(-1) + msqrt(T(1) + sq(a) * t2)) * T(0.5f);
}
template <class T> T ggx_D(V3<T> m, T ax, T ay)
{
    const T c = m.z;
    if (c == T(0))
        return sq(ax) * K<T>::RcpPi;
    const T c2 = sq(c);
    const T s = msqrt(fmx(T(0), T(1) - c2));
    const T c4 = sq(c2);
    const T t2 = (T(1) - c2) / c2;
    const T A = stretched(m, s, ax, ay);
    const T tmp = T(1) + t2 * A;
    return T(1) / (K<T>::Pi * ax * ay * c4 * sq(tmp));
}
template <class T> T ggx_G(V3<T> wi, V3<T> wo, T ax, T ay)
{
    return T(1) / (T(1) + ggx_lambda(wo, ax, ay) + ggx_lambda(wi, ax, ay));
}
template <class T> T ggx_pdf(V3<T> v, V3<T> m, T ax, T ay)
{
    if (v.z == T(0))
        return 0;
    const T G1 = T(1) / (T(1) + ggx_lambda(v, ax, ay));
    return G1 * mfabs(dot(v, m)) * ggx_D(m, ax, ay) / mfabs(v.z);
}
template <class T> V3<T> ggx_sample_m(V3<T> v, T r0, T r1, T ax, T ay)
{
    const T sgn = v.z < T(0) ? T(-1) : T(1);
    const V3<T> st = normalize(v3(sgn * v.x * ax, sgn * v.y * ay, sgn * v.z));
    const V3<T> t1 = v.y < T(0.9999f) ? normalize(cross(st, v3(T(0), T(0), T(1)))) : v3(T(1), T(0), T(0));
    const V3<T> t2 = cross(t1, st);
    const T a = T(1) / (T(1) + st.z);
    const T r = msqrt(r0);
    const T phi = r1 < a ? r1 / a * K<T>::Pi : K<T>::Pi + (r1 - a) / (T(1) - a) * K<T>::Pi;
    T sp, cp;
    sincosT(phi, sp, cp);
    const T p1 = r * cp;
    const T p2 = r * sp * (r1 < a ? T(1) : st.z);
    const V3<T> h = p1 * t1 + p2 * t2 + msqrt(fmx(T(0), T(1) - p1 * p1 - p2 * p2)) * st;
    return normalize(v3(h.x * ax, h.y * ay, fmx(T(0), h.z)));
}
template <class T> T gtr1_lambda(V3<T> v, T ax)
{
    const T c = v.z;
    if (c == T(0))
        return 0;
    const T c2 = sq(c);
    const T s = msqrt(fmx(T(0), T(1) - c2));
    if (s == T(0))
        return 0;
    const T cot2 = c2 / sq(s);
    const T cot = msqrt(cot2);
    const T alpha = clampT(ax, T(0.001f), T(0.999f));
    const T a2 = sq(alpha);
    const T a = msqrt(cot2 + a2);
    const T b = msqrt(cot2 + T(1));
    const T lc = mlog(cot + b);
    const T ld = mlog(cot + a);
    return (a - b + cot * (lc - ld)) / (cot * mlog(a2));
}
template <class T> T gtr1_D(V3<T> m, T ax)
{
    const T alpha = clampT(ax, T(0.001f), T(0.999f));
    const T a2 = sq(alpha);
    const T c2 = sq(m.z);
    const T a = (a2 - T(1)) / (K<T>::Pi * mlog(a2));
    const T b = T(1) / (T(1) + (a2 - T(1)) * c2);
    return a * b;
}
template <class T> T gtr1_G(V3<T> wi, V3<T> wo, T ax) { return T(1) / (T(1) + gtr1_lambda(wo, ax) + gtr1_lambda(wi, ax)); }
template <class T> T gtr1_pdf(V3<T> m, T ax) { return gtr1_D(m, ax) * mfabs(m.y); }
template <class T> V3<T> gtr1_sample_m(T r0, T r1, T ax)
{
    const T alpha = clampT(ax, T(0.001f), T(0.999f));
    const T a2 = sq(alpha);
    const T a = T(1) - std::pow(a2, T(1) - r0);
    const T c2 = a / (T(1) - a2);
    const T c = msqrt(c2);
    const T s = msqrt(fmx(T(0), T(1) - c2));
    T sp, cp;
    sincosT(K<T>::TwoPi * r1, sp, cp);
    return v3(cp * s, sp * s, c);
}

// Disney.h:30-579
template <class T> T schlick(T u)
{
    const T m = saturate(T(1) - u);
    const T m2 = sq(m);
    return sq(m2) * m;
}
template <class T> V3<T> spec_fresnel(const HitMat<T>& mat, V3<T> o, V3<T> h)
{
    V3<T> v = (T(1) - mat.specularTint) + (mat.specularTint * mat.tint);
    v = v * (mat.specular * T(0.08f));
    v = ((T(1) - mat.metallic) * v) + (mat.metallic * mat.diffuse);
    const T f = schlick(mfabs(dot(o, h)));
    return ((T(1) - f) * v) + f;
}
template <class T> V3<T> cc_fresnel(const HitMat<T>& mat, V3<T> o, V3<T> h)
{
    const T f = schlick(mfabs(dot(o, h)));
    return v3s(mix(T(0.04f), T(1), f) * T(0.25f) * mat.clearcoat);
}
template <class T> bool force_above(V3<T>& d)
{
    const T corr = T(1.0e-4f) - d.z;
    if (corr <= 0)
        return false;
    d = normalize(d + corr * v3(T(0), T(0), T(1)));
    return true;
}
template <class T> T d_diffuse(const HitMat<T>& mat, V3<T> wo, V3<T> wi, V3<T>& value)
{
    const V3<T> h = normalize(wi + wo);
    const T con = wo.z, cin = wi.z, cih = dot(wi, h);
    const T fl = schlick(cin), fv = schlick(con);
    T fd = 0;
    if (mat.subsurface != T(1)) {
        const T fd90 = T(0.5f) + T(2) * sq(cih) * mat.roughness;
        fd = mix(T(1), fd90, fl) * mix(T(1), fd90, fv);
    }
    if (mat.subsurface > T(0)) {
        const T fss90 = sq(cih) * mat.roughness;
        const T fss = mix(T(1), fss90, fl) * mix(T(1), fss90, fv);
        const T ss = T(1.25f) * (fss * (T(1) / (mfabs(con) + mfabs(cin)) - T(0.5f)) + T(0.5f));
        fd = mix(fd, ss, mat.subsurface);
    }
    value = mat.diffuse * (fd * K<T>::RcpPi * (T(1) - mat.metallic));
    return mfabs(cin) * K<T>::RcpPi;
}
template <class T> T d_sheen(const HitMat<T>& mat, V3<T> wo, V3<T> wi, V3<T>& value)
{
    const V3<T> h = normalize(wi + wo);
    const T fh = schlick(dot(wi, h));
    value = (T(1) - mat.sheenTint) + (mat.sheenTint * mat.tint);
    value = value * (fh * mat.sheen * (T(1) - mat.metallic));
    return K<T>::RcpTwoPi;
}
template <class T> T d_ggx_eval(T ax, T ay, const HitMat<T>& mat, V3<T> wo, V3<T> wi, V3<T>& value)
{
    if (wo.z == T(0) || wi.z == T(0))
        return 0;
    const V3<T> m = normalize(wi + wo);
    const T coh = dot(wo, m);
    if (coh == T(0))
        return 0;
    const T D = ggx_D(m, ax, ay);
    const T G = ggx_G(wi, wo, ax, ay);
    value = spec_fresnel(mat, wo, m);
    value = value * (D * G / mfabs(T(4) * wo.z * wi.z));
    return ggx_pdf(wo, m, ax, ay) / mfabs(T(4) * coh);
}
template <class T>
void d_ggx_sample(T ax, T ay, const HitMat<T>& mat, T r0, T r1, V3<T> wo, V3<T>& wi, T& pdf, V3<T>& value)
{
    if (wo.z == T(0))
        return;
    V3<T> m = ggx_sample_m(wo, r0, r1, ax, ay);
    wi = reflect(-wo, m);
    if (force_above(wi))
        m = normalize(wo + wi);
    if (wi.z == T(0))
        return;
    const T coh = dot(wo, m);
    pdf = ggx_pdf(wo, m, ax, ay) / mfabs(T(4) * coh);
    if (pdf < T(1e-6f))
        return;
    const T D = ggx_D(m, ax, ay);
    const T G = ggx_G(wi, wo, ax, ay);
    value = spec_fresnel(mat, wo, m);
    value = value * (D * G / mfabs(T(4) * wo.z * wi.z));
}
template <class T> T d_gtr1_eval(T a, const HitMat<T>& mat, V3<T> wo, V3<T> wi, V3<T>& value)
{
    if (wo.z == T(0) || wi.z == T(0))
        return 0;
    const V3<T> m = normalize(wi + wo);
    const T coh = dot(wo, m);
    if (coh == T(0))
        return 0;
    const T D = gtr1_D(m, a);
    const T G = gtr1_G(wi, wo, a);
    value = cc_fresnel(mat, wo, m);
    value = value * (D * G / mfabs(T(4) * wo.z * wi.z));
    return gtr1_pdf(m, a) / mfabs(T(4) * coh);
}
template <class T>
void d_gtr1_sample(T a, const HitMat<T>& mat, T r0, T r1, V3<T> wo, V3<T>& wi, T& pdf, V3<T>& value)
{
    if (wo.z == T(0))
        return;
    V3<T> m = gtr1_sample_m(r0, r1, a);
    wi = reflect(-wo, m);
    if (force_above(wi))
        m = normalize(wo + wi);
    if (wi.z == T(0))
        return;
    const T coh = dot(wo, m);
    pdf = gtr1_pdf(m, a) / mfabs(T(4) * coh);
    if (pdf < T(1e-6f))
        return;
    const T D = gtr1_D(m, a);
    const T G = gtr1_G(wi, wo, a);
    value = spec_fresnel(mat, wo, m);
    value = value * (D * G / mfabs(T(4) * wo.z * wi.z));
}
template <class T> bool d_weights(const HitMat<T>& m, T& wd, T& ws, T& wsp, T& wc)
{
    wd = lerp(m.luminance, T(0), m.metallic);
    ws = lerp(m.sheen, T(0), m.metallic);
    wsp = lerp(m.specular, T(1), m.metallic);
    wc = m.clearcoat * T(0.25f);
    const T total = wd + ws + wsp + wc;
    if (total == T(0))
        return false;
    const T rcp = T(1) / total;
    wd = wd * rcp;
    ws = ws * rcp;
    wsp = wsp * rcp;
    wc = wc * rcp;
    return true;
}
template <class T> T cc_alpha(const HitMat<T>& m) { return mix(T(0.1f), T(0.001f), m.clearcoatGloss); }

template <class T, bool REF> Lobe<T> d_evaluate(V3<T> wo, V3<T> wi, const HitMat<T>& m)
{
    Lobe<T> r{wi, T(0), v3s(T(0)), 0};
    T wd, ws, wsp, wc;
    if (!d_weights(m, wd, ws, wsp, wc))
        return r;
    T pdf = 0;
    V3<T> inc = v3s(T(0));
    if (REF) {
        if (wd > 0) pdf = pdf + wd * d_diffuse(m, wo, wi, inc);
        if (ws > 0) pdf = pdf + ws * d_sheen(m, wo, wi, inc);
    } else {
        V3<T> v = v3s(T(0));
        if (wd > 0) { pdf = pdf + wd * d_diffuse(m, wo, wi, v); inc = inc + v; }
        if (ws > 0) { pdf = pdf + ws * d_sheen(m, wo, wi, v); inc = inc + v; }
    }
    if (wsp > 0) {
        T ax, ay;
        alpha_xy(m.roughness, m.anisotropic, ax, ay);
        V3<T> v = v3s(T(0));
        const T p = d_ggx_eval(ax, ay, m, wo, wi, v);
        if (p > 0) { pdf = pdf + wsp * p; inc = inc + v; }
    }
    if (wc > 0) {
        V3<T> v = v3s(T(0));
        const T p = d_gtr1_eval(cc_alpha(m), m, wo, wi, v);
        if (p > 0) { pdf = pdf + wc * p; inc = inc + v; }
    }
    r.pdf = pdf;
    r.Tv = inc;
    return r;
}

template <class T, bool REF> Lobe<T> d_sample(V3<T> wo, const HitMat<T>& m, T r0, T r1)
{
    Lobe<T> r{v3(T(0), T(0), T(1)), T(0), v3s(T(0)), 0};
    T wd, ws, wsp, wc;
    if (!d_weights(m, wd, ws, wsp, wc))
        return r;
    const T cd = wd, cs = cd + ws, csp = cs + wsp;
    V3<T> wi = v3(T(0), T(0), T(1));
    T prob = 0, cpdf = 0;
    V3<T> value = v3s(T(0));
    uint32_t flags = 0;
    if (r0 < cd) {
        const T u = REF ? r0 : r0 / wd;
        wi = cos_hemi(u, r1);
        cpdf = d_diffuse(m, wo, wi, value);
        prob = wd * cpdf;
        wd = 0;
    } else if (r0 < cs) {
        const T u = REF ? r0 : (r0 - cd) / ws;
        wi = cos_hemi(u, r1);
        cpdf = d_sheen(m, wo, wi, value);
        prob = ws * cpdf;
        ws = 0;
        flags |= REF ? kSpec : 0u;
    } else if (r0 < csp) {
        const T u = REF ? r0 : fmn((r0 - cs) / wsp, T(0.99999994f));
        T ax, ay;
        alpha_xy(m.roughness, m.anisotropic, ax, ay);
        d_ggx_sample(ax, ay, m, u, r1, wo, wi, cpdf, value);
        prob = wsp * cpdf;
        wsp = 0;
        flags |= REF ? kSpec : 0u;
    } else {
        const T u = REF ? r0 : fmn((r0 - csp) / wc, T(0.99999994f));
        d_gtr1_sample(cc_alpha(m), m, u, r1, wo, wi, cpdf, value);
        prob = wc * cpdf;
        wc = 0;
        flags |= REF ? kSpec : 0u;
    }
    if (wd > 0) {
        V3<T> v;
        prob = prob + wd * d_diffuse(m, wo, wi, v);
        value = value + v;
    }
    if (ws > 0) {
        V3<T> v;
        prob = prob + ws * d_sheen(m, wo, wi, v);
        value = value + v;
    }
    if (wsp > 0) {
        T ax, ay;
        alpha_xy(m.roughness, m.anisotropic, ax, ay);
        V3<T> v = v3s(T(0));
        prob = prob + wsp * d_ggx_eval(ax, ay, m, wo, wi, v);
        value = value + v;
    }
    if (wc > 0) {
        V3<T> v = v3s(T(0));
        const T p = d_gtr1_eval(cc_alpha(m), m, wo, wi, v);
        if (!REF)
            prob = prob + wc * p;
        value = value + v;
    }
    r.wi = wi;
    r.pdf = prob > T(1e-6f) ? prob : T(0);
    r.Tv = value;
    r.flags = flags;
    return r;
}

// The default sampling mode's Disney closure (the reference's sampling with its
// quirks fixed): the lobe that r0 falls in picks the extend direction (r0
// rescaled into the lobe's interval), and the light direction and the extend
// direction are both evaluated over all lobes - value = sum of the lobe values,
// pdf = sum of weight x lobe pdf, each lobe term as in d_evaluate<T, false>
// (Disney.h:401-470). Same estimator as Disney::Sample + Disney::Evaluate
// (Disney.h:473-565) without their REF quirks.
template <class T> Clos<T> d_closure_default(V3<T> wo, V3<T> wi, V3<T> Tp, const HitMat<T>& m, T r0, T r1)
{
    Lobe<T> e{wi, T(0), v3s(T(0)), 0};
    Lobe<T> s{v3(T(0), T(0), T(1)), T(0), v3s(T(0)), 0};
    T wd, ws, wsp, wc;
    if (d_weights(m, wd, ws, wsp, wc)) {
        T ax, ay;
        alpha_xy(m.roughness, m.anisotropic, ax, ay);
        const T cd = wd, cs = cd + ws, csp = cs + wsp;
        V3<T> d = v3(T(0), T(0), T(1));
        if (r0 < cd) {
            d = cos_hemi(r0 / wd, r1);
        } else if (r0 < cs) {
            d = cos_hemi((r0 - cd) / ws, r1);
        } else if (wo.z != T(0)) {
            const V3<T> h = r0 < csp ? ggx_sample_m(wo, fmn((r0 - cs) / wsp, T(0.99999994f)), r1, ax, ay)
                                     : gtr1_sample_m(fmn((r0 - csp) / wc, T(0.99999994f)), r1, cc_alpha(m));
            d = reflect(-wo, h);
            force_above(d);
        }
        e = d_evaluate<T, false>(wo, wi, m);
        const Lobe<T> q = d_evaluate<T, false>(wo, d, m);
        s.wi = d;
        s.pdf = q.pdf > T(1e-6f) ? q.pdf : T(0);
        s.Tv = q.Tv;
    }
    return finalize(Tp, e, s);
}

// ---------------------------------------------------------------- camera
template <class T, class Rng> void sample_disk(Rng& rng, T& x, T& y)
{
    float ux, uy;
    draw2(rng, is_ref_rng<Rng>() && g_refRightToLeft, ux, uy);
    const T lx = (T(ux) * T(2)) - T(1);
    const T ly = (T(uy) * T(2)) - T(1);
    if (lx == 0 && ly == 0) {
        x = lx;
        y = ly;
        return;
    }
    T theta, r;
    if (mfabs(lx) > mfabs(ly)) {
        r = lx;
        theta = K<T>::PiOver4 * (ly / lx);
    } else {
        r = ly;
        theta = K<T>::PiOver2 - K<T>::PiOver4 * (lx / ly);
    }
    T s, c;
    sincosT(theta, s, c);
    x = r * c;
    y = r * s;
}

// GenerateCameraRay, optix.cu:142-174 (with SampleBokeh :93-112, Distort :117-138)
template <class T, class Rng>
void camera_ray(const tr_camera& cam, T tanFov2, uint32_t W, uint32_t H, int ix, int iy, Rng& rng,
                V3<T>& O, V3<T>& D, T& Tv)
{
    const V3<T> pos = v3(T(cam.position[0]), T(cam.position[1]), T(cam.position[2]));
    const V3<T> side = v3(T(cam.side[0]), T(cam.side[1]), T(cam.side[2]));
    const V3<T> up = v3(T(cam.up[0]), T(cam.up[1]), T(cam.up[2]));
    const V3<T> fwd = v3(T(cam.forward[0]), T(cam.forward[1]), T(cam.forward[2]));
    O = pos;
    D = fwd;
    Tv = 1;
    float ujx, ujy;
    draw2(rng, is_ref_rng<Rng>() && g_refRightToLeft, ujx, ujy);
    const T jx = T(ujx), jy = T(ujy);
    const T rx = T(W), ry = T(H);
    const T aspect = rx / ry;
    T sx = (((T(ix) + jx) / rx) * T(2)) - T(1);
    T sy = (((T(iy) + jy) / ry) * T(2)) - T(1);
    sy = sy / aspect;
    T bx, by;
    if (cam.bokeh_side_count < 3) {
        sample_disk<T>(rng, bx, by);
    } else {
        const int index = int(T(rng.next()) * T(cam.bokeh_side_count));
        const T step = (T(2) * K<T>::Pi) / T(cam.bokeh_side_count);
        T s0, c0, s1, c1;
        sincosT(T(cam.bokeh_rotation) + (T(index) * step), s0, c0);
        sincosT(T(cam.bokeh_rotation) + T(index + 1) * step, s1, c1);
        const T u1 = T(rng.next()), u2 = T(rng.next());
        const T su = msqrt(u1);
        bx = (su * (T(1) - u2)) * c0 + (su * u2) * c1;
        by = (su * (T(1) - u2)) * s0 + (su * u2) * s1;
    }
    const T ccx = bx * T(cam.aperture), ccy = by * T(cam.aperture);
    T lx = (tanFov2 * sx) - (ccx / T(cam.focal_dist));
    T ly = (tanFov2 * sy) - (ccy / T(cam.focal_dist));
    const T dist = T(cam.distortion);
    if (!(lx == 0 && ly == 0) && dist > 0) {
        const T scale = msqrt(lx * lx + ly * ly);
        const T d = (tanFov2 * dist) * T(0.5f);
        const T distorted = (scale * dist * std::atan(d)) / d;
        if (distorted >= K<T>::PiOver2)
            return;
        const T k = std::tan(distorted) / (scale * dist);
        lx = lx * k;
        ly = ly * k;
    }
    D = normalize(fwd + (lx * side) + (ly * up));
    O = pos + (side * ccx) + (up * ccy);
    const T v = fmx(T(0), dot(D, fwd));
    const T v2 = v * v;
    Tv = v2 * v2;
}

// ---------------------------------------------------------------- shade
// tex2D<float4> of a texture described as the reference's (Texture.cpp:107-139):
// bilinear filtering, wrap addressing, normalised coordinates. Restated from the
// CUDA C++ Programming Guide ("Texture Fetching", linear filtering): the
// coordinate is wrapped to [0, 1), scaled by the size, shifted by half a texel;
// the neighbouring texels wrap around the edges and the fractional weights are
// held in fixed point with 8 fractional bits.
void texture_sample(const Texture& t, float u, float v, float out[4])
{
    auto wrap = [](float x) { return std::isfinite(x) ? x - std::floor(x) : 0.f; };
    const float x = wrap(u) * float(t.w) - 0.5f;
    const float y = wrap(v) * float(t.h) - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float a = std::nearbyint((x - fx) * 256.f) * (1.f / 256.f);
    const float b = std::nearbyint((y - fy) * 256.f) * (1.f / 256.f);
    const int64_t W = t.w, H = t.h;
    const int64_t i0 = ((int64_t(fx) % W) + W) % W, j0 = ((int64_t(fy) % H) + H) % H;
    const int64_t i1 = (i0 + 1) % W, j1 = (j0 + 1) % H;
    auto texel = [&](int64_t i, int64_t j, int c) { return hval(t.texels[4 * size_t(j * W + i) + size_t(c)]); };
    for (int c = 0; c < 4; ++c)
        out[c] = ((1.f - a) * (1.f - b)) * texel(i0, j0, c) + (a * (1.f - b)) * texel(i1, j0, c) +
                 ((1.f - a) * b) * texel(i0, j1, c) + (a * b) * texel(i1, j1, c);
}

int32_t material_texture(const orc_scene& S, uint32_t matIx, uint32_t prop)
{
    return S.matTex.empty() ? -1 : S.matTex[size_t(matIx) * TR_PROP_COUNT + prop];
}

// GetColor (CudaMaterial.h:77-95) for the properties with a texture: the stored
// colour times the texture's RGB at uv, in float.
MatRaw textured_raw(const orc_scene& S, uint32_t matIx, float u, float v)
{
    MatRaw r = S.mats[matIx];
    auto tex = [&](uint32_t p, float rgb[3]) {
        const int32_t ti = material_texture(S, matIx, p);
        if (ti < 0)
            return false;
        float o[4];
        texture_sample(S.textures[size_t(ti)], u, v, o);
        rgb[0] = o[0];
        rgb[1] = o[1];
        rgb[2] = o[2];
        return true;
    };
    float c[3];
    if (tex(TR_PROP_DIFFUSE, c))
        for (int k = 0; k < 3; ++k)
            r.diffuse[k] = r.diffuse[k] * c[k];
    const std::pair<uint32_t, float*> scalars[] = {
        {TR_PROP_ANISOTROPIC, &r.anisotropic}, {TR_PROP_CLEARCOAT, &r.clearcoat},
        {TR_PROP_CLEARCOAT_GLOSS, &r.clearcoatGloss}, {TR_PROP_METALLIC, &r.metallic},
        {TR_PROP_ROUGHNESS, &r.roughness}, {TR_PROP_SHEEN, &r.sheen}, {TR_PROP_SHEEN_TINT, &r.sheenTint},
        {TR_PROP_SPECULAR, &r.specular}, {TR_PROP_SPECULAR_TINT, &r.specularTint},
        {TR_PROP_SUBSURFACE, &r.subsurface}};
    for (const auto& sc : scalars)
        if (tex(sc.first, c))
            *sc.second = *sc.second * c[0];
    return r;
}

template <class T>
struct Surface {
    V3<T> N, Ng, Tn, B;
    T area;
    uint32_t matIx;
    float u, v;   // texture coordinate (float, as the reference interpolates it)
};

// GetIntersectionAttributes + FixNormals, CudaMaterial.h:102-212. prim is the
// global triangle index; inst selects the inverse instance transform applied to
// the frame (two-level scenes; one-level scenes have the identity).
template <class T> Surface<T> surface_at(const orc_scene& S, uint32_t prim, T bu, T bv, V3<T> D, uint32_t inst = 0)
{
    const Tri& t = S.tris[prim];
    Surface<T> sf;
    sf.matIx = S.matIdx[prim];
    const V3<T> v0 = v3(T(t.v[0][0]), T(t.v[0][1]), T(t.v[0][2]));
    const V3<T> v1 = v3(T(t.v[1][0]), T(t.v[1][1]), T(t.v[1][2]));
    const V3<T> v2 = v3(T(t.v[2][0]), T(t.v[2][1]), T(t.v[2][2]));
    const V3<T> e1 = v1 - v0, e2 = v2 - v0;
    sf.area = length(cross(e1, e2)) * T(0.5f);
    V3<T> n[3];
    for (int k = 0; k < 3; ++k)
        n[k] = v3(T(hval(t.n[k][0])), T(hval(t.n[k][1])), T(hval(t.n[k][2])));
    sf.N = normalize(n[0] + ((n[1] - n[0]) * bu) + ((n[2] - n[0]) * bv));
    sf.Ng = v3(T(hval(t.N[0])), T(hval(t.N[1])), T(hval(t.N[2])));
    // texcoord: Barycentric of the fp16 texcoords, in float (CudaMaterial.h:131-135)
    {
        const float fu = float(bu), fv = float(bv);
        float uv[3][2];
        for (int k = 0; k < 3; ++k) {
            uv[k][0] = hval(t.uv[k][0]);
            uv[k][1] = hval(t.uv[k][1]);
        }
        sf.u = uv[0][0] + ((uv[1][0] - uv[0][0]) * fu) + ((uv[2][0] - uv[0][0]) * fv);
        sf.v = uv[0][1] + ((uv[1][1] - uv[0][1]) * fu) + ((uv[2][1] - uv[0][1]) * fv);
    }
    const int32_t normalTex = material_texture(S, sf.matIx, TR_PROP_NORMAL);
    if (normalTex >= 0) {
        // normal map applied before the tangent frame exists (CudaMaterial.h:185-191 with the
        // zero tangent and bitangent of a zero-initialised Intersection)
        float o[4];
        texture_sample(S.textures[size_t(normalTex)], sf.u, sf.v, o);
        const V3<T> nm = v3(T(o[0]), T(o[1]), T(o[2]));
        const V3<T> norMap = (nm * T(2)) - v3s(T(1));
        const V3<T> zero = v3s(T(0));
        sf.N = normalize(zero * norMap.x + zero * norMap.y + sf.N * norMap.z);
    }
    // texcoord differences are taken in fp16 (half subtraction)
    const T s1 = T(hround(hval(t.uv[1][0]) - hval(t.uv[0][0])));
    const T t1 = T(hround(hval(t.uv[1][1]) - hval(t.uv[0][1])));
    const T s2 = T(hround(hval(t.uv[2][0]) - hval(t.uv[0][0])));
    const T t2 = T(hround(hval(t.uv[2][1]) - hval(t.uv[0][1])));
    const T r = (s1 * t2) - (s2 * t1);
    if (mfabs(r) < T(1e-6f)) {
        sf.B = normalize(cross(sf.N, e1));
        sf.Tn = normalize(cross(sf.N, sf.B));
    } else {
        const T rr = T(1) / r;
        const V3<T> tv = ((s1 * e2) - (s2 * e1)) * rr;
        sf.B = normalize(tv - sf.N * dot(sf.N, tv));
        sf.Tn = normalize(cross(sf.N, sf.B));
    }
    if (S.twoLevel) {
        // object -> world: transform(tx, ty, tz, v) with the inverse rows, CudaMaterial.h:204-211
        const float* m = &S.instInv[12 * size_t(inst)];
        auto xf = [&](V3<T> v) {
            return v3(dot(v, v3(T(m[0]), T(m[4]), T(m[8]))), dot(v, v3(T(m[1]), T(m[5]), T(m[9]))),
                      dot(v, v3(T(m[2]), T(m[6]), T(m[10]))));
        };
        sf.N = xf(sf.N);
        sf.Ng = xf(sf.Ng);
        sf.B = xf(sf.B);
        sf.Tn = xf(sf.Tn);
    }
    // (one level: the identity inverse instance transform) transform() then normalize
    sf.N = normalize(sf.N);
    sf.Ng = normalize(sf.Ng);
    sf.B = normalize(sf.B);
    sf.Tn = normalize(sf.Tn);
    if (dot(D, sf.N) > T(0)) {
        sf.Ng = -sf.Ng;
        sf.N = -sf.N;
        sf.Tn = -sf.Tn;
        sf.B = -sf.B;
    }
    return sf;
}

// material resolution, CudaMaterial.h:171-183 (LinearToCIEXYZ / CIEXYZToLinear, CudaUtility.h:32-50)
template <class T> HitMat<T> hit_material(const MatRaw& r)
{
    HitMat<T> m;
    m.diffuse = v3(T(r.diffuse[0]), T(r.diffuse[1]), T(r.diffuse[2]));
    const V3<T> d = m.diffuse;
    const V3<T> xyz = v3(fmx(T(0), T(0.412453f) * d.x + T(0.357580f) * d.y + T(0.180423f) * d.z),
                         fmx(T(0), T(0.212671f) * d.x + T(0.715160f) * d.y + T(0.072169f) * d.z),
                         fmx(T(0), T(0.019334f) * d.x + T(0.119193f) * d.y + T(0.950227f) * d.z));
    m.metallic = T(r.metallic);
    m.emissive = v3(T(r.emissive[0]), T(r.emissive[1]), T(r.emissive[2])) * m.diffuse;
    m.subsurface = T(r.subsurface);
    if (xyz.y > T(0)) {
        const V3<T> x = xyz * (T(1) / xyz.y);
        m.tint = v3(fmx(T(0), T(3.240479f) * x.x - T(1.537150f) * x.y - T(0.498535f) * x.z),
                    fmx(T(0), T(-0.969256f) * x.x + T(1.875992f) * x.y + T(0.041556f) * x.z),
                    fmx(T(0), T(0.055648f) * x.x - T(0.204043f) * x.y + T(1.057311f) * x.z));
    } else {
        m.tint = v3s(T(1));
    }
    m.specular = T(r.specular);
    m.roughness = T(r.roughness);
    m.specularTint = T(r.specularTint);
    m.anisotropic = T(r.anisotropic);
    m.sheen = T(r.sheen);
    m.sheenTint = T(r.sheenTint);
    m.clearcoat = T(r.clearcoat);
    m.clearcoatGloss = T(r.clearcoatGloss);
    m.luminance = xyz.y;
    m.closure = r.closure;
    return m;
}

// SafeColor / fixnan, CudaUtility.h:95-99, CudaLinearMath.h:127-142
template <class T> V3<T> safe_color(V3<T> c, T maxValue)
{
    V3<T> r = c;
    const T m = std::fmax(c.x, std::fmax(c.y, c.z));
    if (!(m <= maxValue))
        r = c * (maxValue / m);
    return finite3(r) ? r : v3s(T(0));
}
template <class T> V3<T> fixnan(V3<T> c) { return finite3(c) ? c : v3s(T(0)); }

template <class T> struct ShadeOut {
    bool ext = false, sh = false;
    V3<T> extO, extD, extT;
    T extPdf = 0;
    uint32_t extPacked = 0;
    uint32_t extNormal = 0;
    V3<T> shO, shL, shT;
    T shDist = 0;
    V3<T> add = v3s(T(0));
    // vertex data for the adjoint
    bool hit = false, emissive = false;
    uint32_t matIx = 0;
    int lightIx = -1;
    V3<T> wo, wiLight, wiExt;
};

// SampleLight / SelectLight, CudaLights.h:38-124
template <class T, bool REF, class Rng>
V3<T> sample_light(const orc_scene& S, Rng& rng, V3<T> I, V3<T> N, T& prob, T& pdf, V3<T>& rad, T& dist,
                   int* lightOut = nullptr)
{
    const float total = REF ? S.lightEnergy : S.lightEnergyTotal;
    const int32_t count = int32_t(S.lights.size());
    if (total == 0 || count == 0) {
        prob = 0;
        pdf = 0;
        rad = v3s(T(0));
        dist = T(1e20f);
        return v3(T(0), T(1), T(0));
    }
    int32_t ix = -1;
    V3<T> P;
    if (REF) {
        const float e = rng.next() * S.lightEnergy;
        int32_t low = 0, high = count - 1;
        for (int it = 0; it < 64 && low <= high; ++it) {
            const int32_t mid = (low + high) >> 1;
            const Light& L = S.lights[mid];
            if (e < L.sumEnergy)
                high = mid;
            else if (e > L.sumEnergy + L.energy)
                low = mid + 1;
            else {
                ix = mid;
                break;
            }
        }
        if (ix < 0) {
            const int c = int(rng.next() * float(count));
            ix = std::max(0, std::min(c, count - 1));
        }
        const Light& L = S.lights[ix];
        float u0, u1, u2;
        draw3(rng, g_refRightToLeft, u0, u1, u2);
        const T b0 = T(u0), b1 = T(u1), b2 = T(u2);
        P = (b0 * v3(T(L.V0[0]), T(L.V0[1]), T(L.V0[2]))) + (b1 * v3(T(L.V1[0]), T(L.V1[1]), T(L.V1[2]))) +
            (b2 * v3(T(L.V2[0]), T(L.V2[1]), T(L.V2[2])));
    } else {
        const float u = rng.next();
        const float coin = rng.next();
        uint32_t k = uint32_t(u * float(count));
        k = k < uint32_t(count) ? k : uint32_t(count) - 1u;
        ix = int32_t(coin < S.alias[k].prob ? k : S.alias[k].alias);
        const Light& L = S.lights[ix];
        const T r0 = T(rng.next()), r1 = T(rng.next());
        const T su = msqrt(r0);
        P = ((T(1) - su) * v3(T(L.V0[0]), T(L.V0[1]), T(L.V0[2]))) +
            ((su * (T(1) - r1)) * v3(T(L.V1[0]), T(L.V1[1]), T(L.V1[2]))) +
            ((su * r1) * v3(T(L.V2[0]), T(L.V2[1]), T(L.V2[2])));
    }
    if (lightOut)
        *lightOut = ix;
    const Light& L = S.lights[ix];
    V3<T> Ld = I - P;
    const T sqDist = dot(Ld, Ld);
    Ld = normalize(Ld);
    const V3<T> LN = v3(T(L.N[0]), T(L.N[1]), T(L.N[2]));
    const T LNdotL = dot(LN, Ld);
    prob = T(L.energy) / T(total);
    const bool facing = REF ? (dot(N, Ld) != T(0)) : (dot(N, Ld) < T(0));
    pdf = (LNdotL > 0 && facing) ? sqDist / (T(L.area) * LNdotL) : T(0);
    dist = msqrt(sqDist);
    rad = v3(T(L.radiance[0]), T(L.radiance[1]), T(L.radiance[2]));
    return -Ld;
}

// SampleSky, CudaSky.h:105-156 (Preetham sky), every term evaluated per call in T
// as the reference does; black when the sky is disabled.
template <class T>
V3<T> sample_sky(const orc_scene& S, V3<T> D, bool drawSun)
{
    using std::acos;
    using std::cos;
    using std::exp;
    using std::pow;
    const auto& k = S.sky;
    if (k.enabled == 0)
        return v3s(T(0));
    const T Pi = K<T>::Pi;
    const V3<T> sunDir = v3(T(k.sunDir[0]), T(k.sunDir[1]), T(k.sunDir[2]));
    const T cosAD = T(k.cosSunAngularDiameter);
    const V3<T> up = v3(T(0), T(1), T(0));
    const T cosSunUp = dot(sunDir, up);
    auto sat = [](T x) { return x < T(0) ? T(0) : (x > T(1) ? T(1) : x); };
    T sunfade = T(1) - sat(T(1) - exp(-sunDir.z / T(500)));
    const T rayleigh = T(2.5f) - (T(1) * (T(1) - sunfade));
    const T lambda[3] = {T(620e-9f), T(492e-9f), T(390e-9f)};
    const T K[3] = {T(0.686f), T(0.678f), T(0.666f)};
    const T num = T(8) * pow(Pi, T(3)) * pow(pow(T(1.0003f), T(2)) - T(1), T(2)) * (T(6) + T(3) * T(0.031f));
    const T c = T(0.2f) * T(k.turbidity) * T(10e-18f);
    T bR[3], bM[3];
    for (int i = 0; i < 3; ++i) {
        bR[i] = (num / ((T(3) * T(2.545e25f)) * pow(lambda[i], T(4)) * (T(6) - T(7) * T(0.031f)))) * rayleigh;
        bM[i] = (T(0.434f) * c * Pi * pow((T(2) * Pi) / lambda[i], T(4) - T(2)) * K[i]) * T(0.005f);
    }
    const T zenith = acos(std::max(dot(up, D), T(0)));
    const T denom = cos(zenith) + T(0.15f) * pow(T(93.885f) - ((zenith * T(180)) / Pi), T(-1.253f));
    const T sR = T(8.4e3f) / denom, sM = T(1.25e3f) / denom;
    const T cosTheta = dot(D, sunDir);
    const T rPhase = (T(3) / (T(16) * Pi)) * (T(1) + pow(cosTheta * T(0.5f) + T(0.5f), T(2)));
    const T g = T(0.80f);
    const T hg = (T(1) / (T(4) * Pi)) * ((T(1) - pow(g, T(2))) / pow(T(1) - T(2) * g * cosTheta + pow(g, T(2)), T(1.5f)));
    const T sunE = T(k.sunIntensity) *
                   std::max(T(0), T(1) - exp(-(((Pi / T(1.95f)) - acos(cosSunUp)) / T(1.5f))));
    const T hmix = sat(pow(T(1) - cosSunUp, T(5)));
    const T e0 = cosAD, e1 = cosAD + T(2e-5f);
    const T y = std::max(T(0), std::min((cosTheta - e0) / (e1 - e0), T(1)));
    const T sundisk = y * y * (T(3) - (T(2) * y));
    T Fex[3], Lin[3], L0[3];
    for (int i = 0; i < 3; ++i) {
        Fex[i] = exp(-(bR[i] * sR + bM[i] * sM));
        const T ratio = ((bR[i] * rPhase) + (bM[i] * hg)) / (bR[i] + bM[i]);
        Lin[i] = pow((sunE * ratio) * (T(1) - Fex[i]), T(1.5f));
        Lin[i] = Lin[i] * ((T(1) * (T(1) - hmix)) + (pow((sunE * ratio) * Fex[i], T(0.5f)) * hmix));
        L0[i] = (T(0.1f) * Fex[i]) + ((((sunE * T(19000)) * Fex[i]) * sundisk) * (drawSun ? T(1) : T(0)));
    }
    const T luma = L0[0] * T(0.299f) + L0[1] * T(0.587f) + L0[2] * T(0.114f);
    const T t = std::max(sunDir.y, T(0));
    sunfade = sunfade * ((T(1) * (T(1) - t)) + (T(0.9f) * t));
    const T expo = T(1) / (T(1) + sunfade);
    T out[3];
    for (int i = 0; i < 3; ++i) {
        const T l0 = (luma * (T(1) - T(0.5f))) + (L0[i] * T(0.5f));
        const T cc = Lin[i] + l0;
        const T tm = (cc * (T(1) + cc / T(1000))) / (cc + T(128));
        out[i] = pow(std::max(T(0), tm), expo);
    }
    return v3(out[0], out[1], out[2]);
}

// PathTracingKernel body, PathTracing.h:15-174
template <class T, bool REF, class Rng>
ShadeOut<T> shade_one(const orc_scene& S, const tr_kernel_settings& st, uint32_t bounce, V3<T> O, V3<T> D,
                      V3<T> Tp, T extendPdf, uint32_t pathIx, uint32_t flags, uint32_t primIx, T bu, T bv, T tmax,
                      Rng& rng, uint32_t inst = 0)
{
    ShadeOut<T> out;
    const T maxColor = T(st.max_color > 0.f ? st.max_color : 10.f);
    const V3<T> I = O + D * tmax;
    if (primIx == 0xffffffffu) {
        // PathTracing.h:40-55: T * SampleSky, the sun disc for camera and specular paths
        if (S.sky.enabled) {
            const bool sun = S.sky.drawSun != 0.f && (bounce == 0 || (flags & 1u));
            out.add = safe_color<T>(Tp * sample_sky<T>(S, D, sun), maxColor);
        }
        return out;
    }
    const Surface<T> sf = surface_at<T>(S, primIx, bu, bv, D, inst);
    const HitMat<T> m = S.matTex.empty() ? hit_material<T>(S.mats[sf.matIx])
                                         : hit_material<T>(textured_raw(S, sf.matIx, sf.u, sf.v));
    out.hit = true;
    out.matIx = sf.matIx;
    if (m.emissive.x + m.emissive.y + m.emissive.z > T(kEps)) {
        out.emissive = true;
        V3<T> contrib = v3s(T(0));
        if (bounce == 0 || (flags & kSpec)) {
            contrib = m.emissive;
        } else {
            const T lightPdf = (tmax * tmax) / (mfabs(dot(D, sf.N)) * sf.area);
            const V3<T> en = m.emissive * sf.area;
            const T total = T(REF ? S.lightEnergy : S.lightEnergyTotal);
            const T pick = (en.x + en.y + en.z) / total;
            const T denom = extendPdf + lightPdf * pick;
            if (REF) {
                if (denom > 0)
                    contrib = Tp * m.diffuse * (T(1) / denom);
            } else {
                if (denom > 0)
                    contrib = Tp * m.emissive * (extendPdf / denom);
            }
        }
        out.add = safe_color(contrib, maxColor);
        if (REF && bounce == 0)
            out.add = out.add + m.emissive;
        return out;
    }

    T lightProb, lightPdf, lightDist;
    V3<T> lightRad;
    const V3<T> L = sample_light<T, REF>(S, rng, I, sf.N, lightProb, lightPdf, lightRad, lightDist, &out.lightIx);
    const V3<T> wow = -D;
    const V3<T> wo = normalize(v3(dot(wow, sf.Tn), dot(wow, sf.B), dot(wow, sf.N)));
    const V3<T> wi = normalize(v3(dot(L, sf.Tn), dot(L, sf.B), dot(L, sf.N)));
    float u0, u1;
    draw2(rng, REF && g_refRightToLeft, u0, u1);
    const T r0 = T(u0);
    const T r1 = T(u1);
    Clos<T> c;
    if (m.closure == TR_CLOSURE_DISNEY)
        c = REF ? finalize(Tp, d_evaluate<T, true>(wo, wi, m), d_sample<T, true>(wo, m, r0, r1))
                : d_closure_default<T>(wo, wi, Tp, m, r0, r1);
    else if (m.closure == TR_CLOSURE_DIFFUSE)
        c = diffuse(wo, wi, Tp, m, r0, r1);
    else
        c = lambert(wo, wi, Tp, m, r0, r1);

    if ((lightPdf > T(kEps)) && (c.shPdf > T(kEps)) && ((c.extFlags & kSpec) == 0)) {
        const V3<T> shadowT = (c.shT * lightRad) / (lightProb * lightPdf + c.shPdf);
        out.sh = true;
        out.shO = I;
        out.shL = L;
        out.shDist = lightDist;
        out.shT = safe_color(shadowT, maxColor);
    }
    out.wo = wo;
    out.wiLight = wi;
    out.wiExt = c.extWi;
    if (c.extPdf > T(kEps)) {
        V3<T> tp = c.extT / mfabs(c.extPdf);
        if (bounce >= st.rr_start) {
            const T rr = fmn(T(1), fmx(tp.x, fmx(tp.y, tp.z)));
            if (rr < T(rng.next()))
                return out;
            tp = tp * (T(1) / rr);
        }
        const V3<T> nd = normalize((c.extWi.x * sf.Tn) + (c.extWi.y * sf.B) + (c.extWi.z * sf.N));
        uint32_t fl = flags;
        if (c.extFlags & kSpec)
            fl |= kSpec;
        else
            fl &= ~kSpec;
        out.ext = true;
        out.extO = I;
        out.extD = nd;
        out.extT = fixnan(tp);
        out.extPdf = c.extPdf;
        out.extPacked = (pathIx << 4) | (fl & 15u);
        auto sat16 = [](T x) -> uint32_t {
            const double y = double(float(x * T(65535.f)));
            return y <= 0 ? 0u : (y >= 4294967295.0 ? 0xffffffffu : uint32_t(y));
        };
        out.extNormal = (sat16(sf.N.x) << 16) | sat16(sf.N.y);
    }
    return out;
}

inline uint32_t encode_bary(float u, float v)
{
    const uint32_t bx = static_cast<uint32_t>(u * 65535.f) & 0xFFFFu;
    const uint32_t by = static_cast<uint32_t>(v * 65535.f) & 0xFFFFu;
    return (bx << 16) | by;
}

template <class T> inline T decode16(uint32_t b) { return T(static_cast<float>(b) / 65535.f); }

// One path, depth first: generate, then per bounce closest hit, shade, shadow ray.
template <class T, bool REF>
V3<T> render_path(const orc_scene& S, const tr_camera& cam, T tanFov2, const tr_kernel_settings& st, uint32_t W,
                  uint32_t H, uint32_t sampleCount, uint32_t pathIx, uint64_t& nExt, uint64_t& nSh)
{
    const uint32_t wh = W * H;
    const uint32_t pixel = pathIx % wh;
    V3<T> O, D;
    T Tv;
    if (REF) {
        RefRng rng{tea2(st.seed + pathIx, sampleCount << 1)};
        camera_ray<T>(cam, tanFov2, W, H, pixel % W, pixel / W, rng, O, D, Tv);
    } else {
        CounterRng rng{pixel, sampleCount + pathIx / wh, 0u, st.seed};
        camera_ray<T>(cam, tanFov2, W, H, pixel % W, pixel / W, rng, O, D, Tv);
    }
    V3<T> Tp = v3s(Tv);
    T extendPdf = 1;
    uint32_t flags = 0;
    V3<T> radiance = v3s(T(0));
    const T eps = T(st.ray_epsilon);
    for (uint32_t b = 0; b < st.max_depth; ++b) {
        ++nExt;
        T tmax = T(kDstMax);
        uint32_t prim = 0xffffffffu, inst = 0;
        T bu = 0, bv = 0;
        const T Oa[3] = {O.x, O.y, O.z}, Da[3] = {D.x, D.y, D.z};
        if (!trace<T>(S, Oa, Da, eps, tmax, false, prim, bu, bv, &inst)) {
            prim = 0xffffffffu;
            tmax = T(kDstMax);
        }
        T u16 = 0, v16 = 0;
        if (prim != 0xffffffffu) {
            // the hit record carries 16-bit barycentrics (optix.cu:39-44 / CudaUtility.h:130-146)
            const uint32_t eb = encode_bary(float(bu), float(bv));
            u16 = decode16<T>(eb >> 16);
            v16 = decode16<T>(eb & 0xFFFFu);
        }
        ShadeOut<T> so;
        if (REF) {
            RefRng rng{tea2(st.seed + pathIx, sampleCount + b + 1u)};
            so = shade_one<T, true>(S, st, b, O, D, Tp, extendPdf, pathIx, flags, prim, u16, v16, tmax, rng, inst);
        } else {
            CounterRng rng{pixel, sampleCount + pathIx / wh, b + 1u, st.seed};
            so = shade_one<T, false>(S, st, b, O, D, Tp, extendPdf, pathIx, flags, prim, u16, v16, tmax, rng, inst);
        }
        radiance = radiance + so.add;
        if (so.sh) {
            ++nSh;
            T smax = so.shDist - T(2) * eps;
            uint32_t p2 = 0;
            T a, c;
            const T So[3] = {so.shO.x, so.shO.y, so.shO.z}, Sd[3] = {so.shL.x, so.shL.y, so.shL.z};
            if (!trace<T>(S, So, Sd, eps, smax, true, p2, a, c))
                radiance = radiance + so.shT;
        }
        if (!so.ext)
            break;
        O = so.extO;
        D = so.extD;
        Tp = so.extT;
        extendPdf = so.extPdf;
        flags = so.extPacked & 15u;
    }
    return radiance;
}


// ---------------------------------------------------------------- adjoint
// Path-replay gradient of one path (default sampling mode): the path is
// traced once recording each vertex's contributions, then the closure value
// at every vertex is differentiated (dual numbers) and weighted by the
// radiance that went through it: its own NEE contribution for the light
// direction, the sum of all later contributions for the extend direction.
// Sampled directions, pdfs and MIS weights are held fixed.
template <class T>
struct VertexRec {
    ShadeOut<T> so;
    bool visible = false;
    V3<T> cNee = v3s(T(0));
};

template <class T>
V3<DualT<double>> dual_value(const orc_scene& S, uint32_t matIx, V3<T> wo, V3<T> wi)
{
    using D = DualT<double>;
    const MatRaw& r = S.mats[matIx];
    // seed the six parameters, then resolve tint/luminance with duals (CudaMaterial.h:155-183)
    MatRaw rr = r;
    HitMat<D> m = hit_material<D>(rr);
    m.diffuse = v3(D::var(r.diffuse[0], 0), D::var(r.diffuse[1], 1), D::var(r.diffuse[2], 2));
    {
        const V3<D> d = m.diffuse;
        const V3<D> xyz = v3(fmx(D(0.0), D(0.412453f) * d.x + D(0.357580f) * d.y + D(0.180423f) * d.z),
                             fmx(D(0.0), D(0.212671f) * d.x + D(0.715160f) * d.y + D(0.072169f) * d.z),
                             fmx(D(0.0), D(0.019334f) * d.x + D(0.119193f) * d.y + D(0.950227f) * d.z));
        if (xyz.y > 0) {
            const V3<D> x = xyz * (D(1.0) / xyz.y);
            m.tint = v3(fmx(D(0.0), D(3.240479f) * x.x - D(1.537150f) * x.y - D(0.498535f) * x.z),
                        fmx(D(0.0), D(-0.969256f) * x.x + D(1.875992f) * x.y + D(0.041556f) * x.z),
                        fmx(D(0.0), D(0.055648f) * x.x - D(0.204043f) * x.y + D(1.057311f) * x.z));
        } else {
            m.tint = v3s(D(1.0));
        }
        m.luminance = xyz.y;
    }
    m.roughness = D::var(r.roughness, 3);
    m.metallic = D::var(r.metallic, 4);
    m.specular = D::var(r.specular, 5);
    const V3<D> o = v3(D(double(wo.x)), D(double(wo.y)), D(double(wo.z)));
    const V3<D> i = v3(D(double(wi.x)), D(double(wi.y)), D(double(wi.z)));
    if (r.closure == TR_CLOSURE_DIFFUSE)
        return m.diffuse * K<D>::RcpPi;
    if (r.closure != TR_CLOSURE_DISNEY)
        return v3s(D(0.0));
    return d_evaluate<D, false>(o, i, m).Tv;
}

template <class T>
void adjoint_path(const orc_scene& S, const tr_camera& cam, T tanFov2, const tr_kernel_settings& st, uint32_t W,
                  uint32_t H, uint32_t sampleCount, uint32_t pathIx, const double delta[3], double* grads)
{
    const uint32_t wh = W * H;
    const uint32_t pixel = pathIx % wh;
    V3<T> O, D;
    T Tv;
    {
        CounterRng rng{pixel, sampleCount + pathIx / wh, 0u, st.seed};
        camera_ray<T>(cam, tanFov2, W, H, pixel % W, pixel / W, rng, O, D, Tv);
    }
    V3<T> Tp = v3s(Tv);
    T extendPdf = 1;
    uint32_t flags = 0;
    const T eps = T(st.ray_epsilon);
    std::vector<VertexRec<T>> verts;
    for (uint32_t b = 0; b < st.max_depth; ++b) {
        T tmax = T(kDstMax);
        uint32_t prim = 0xffffffffu, inst = 0;
        T bu = 0, bv = 0;
        const T Oa[3] = {O.x, O.y, O.z}, Da[3] = {D.x, D.y, D.z};
        if (!trace<T>(S, Oa, Da, eps, tmax, false, prim, bu, bv, &inst)) {
            prim = 0xffffffffu;
            tmax = T(kDstMax);
        }
        T u16 = 0, v16 = 0;
        if (prim != 0xffffffffu) {
            const uint32_t eb = encode_bary(float(bu), float(bv));
            u16 = decode16<T>(eb >> 16);
            v16 = decode16<T>(eb & 0xFFFFu);
        }
        CounterRng rng{pixel, sampleCount + pathIx / wh, b + 1u, st.seed};
        VertexRec<T> vr;
        vr.so = shade_one<T, false>(S, st, b, O, D, Tp, extendPdf, pathIx, flags, prim, u16, v16, tmax, rng, inst);
        if (vr.so.sh) {
            T smax = vr.so.shDist - T(2) * eps;
            uint32_t p2 = 0;
            T a, c;
            const T So[3] = {vr.so.shO.x, vr.so.shO.y, vr.so.shO.z}, Sd[3] = {vr.so.shL.x, vr.so.shL.y, vr.so.shL.z};
            vr.visible = !trace<T>(S, So, Sd, eps, smax, true, p2, a, c);
            if (vr.visible)
                vr.cNee = vr.so.shT;
        }
        verts.push_back(vr);
        if (!vr.so.ext)
            break;
        O = vr.so.extO;
        D = vr.so.extD;
        Tp = vr.so.extT;
        extendPdf = vr.so.extPdf;
        flags = vr.so.extPacked & 15u;
    }
    // suffix sums of the contributions after each vertex
    const size_t n = verts.size();
    std::vector<V3<double>> after(n + 1, v3(0.0, 0.0, 0.0));
    for (size_t k = n; k-- > 0;) {
        const V3<T>& a = verts[k].so.add;
        after[k] = after[k + 1] + v3(double(a.x) + double(verts[k].cNee.x), double(a.y) + double(verts[k].cNee.y),
                                     double(a.z) + double(verts[k].cNee.z));
    }
    for (size_t k = 0; k < n; ++k) {
        const VertexRec<T>& vr = verts[k];
        if (!vr.so.hit)
            break;
        double* g = grads + size_t(vr.so.matIx) * 9;
        if (vr.so.emissive) {
            // emission = Emissive * diffuse (CudaMaterial.h:158): linear in both
            const MatRaw& mr = S.mats[vr.so.matIx];
            const double C[3] = {double(vr.so.add.x), double(vr.so.add.y), double(vr.so.add.z)};
            for (int c = 0; c < 3; ++c) {
                if (mr.emissive[c] > 0)
                    g[6 + c] += delta[c] * C[c] / double(mr.emissive[c]);
                if (mr.diffuse[c] > 0)
                    g[c] += delta[c] * C[c] / double(mr.diffuse[c]);
            }
            break;
        }
        auto accumulate = [&](const V3<T>& wi, const double w[3]) {
            const V3<DualT<double>> f = dual_value<T>(S, vr.so.matIx, vr.so.wo, wi);
            const DualT<double>* fc[3] = {&f.x, &f.y, &f.z};
            for (int c = 0; c < 3; ++c)
                if (w[c] != 0.0 && fc[c]->v != 0.0)
                    for (int p = 0; p < kDP; ++p)
                        g[p] += w[c] * fc[c]->d[p] / fc[c]->v;
        };
        if (vr.visible) {
            const double w[3] = {delta[0] * double(vr.cNee.x), delta[1] * double(vr.cNee.y),
                                 delta[2] * double(vr.cNee.z)};
            accumulate(vr.so.wiLight, w);
            if (vr.so.lightIx >= 0) {
                const Light& L = S.lights[size_t(vr.so.lightIx)];
                double* ge = grads + size_t(S.matIdx[size_t(L.triIx)]) * 9;
                for (int c = 0; c < 3; ++c)
                    if (L.radiance[c] > 0)
                        ge[6 + c] += w[c] / double(L.radiance[c]);
            }
        }
        if (vr.so.ext) {
            const double w[3] = {delta[0] * after[k + 1].x, delta[1] * after[k + 1].y, delta[2] * after[k + 1].z};
            accumulate(vr.so.wiExt, w);
        }
    }
}

template <class T>
void shade_entries(const orc_scene* s, const tr_kernel_settings* st, uint32_t bounce, uint32_t sc, uint32_t W,
                   uint32_t H, uint32_t n, const float* O4, const float* D4, const float* T4, const uint32_t* hits,
                   float* ext, uint8_t* ext_valid, float* sh, uint8_t* sh_valid, float* radiance_add)
{
    const uint32_t wh = W * H;
    const bool ref = st->flags & TR_FLAG_REFERENCE_SAMPLING;
    for (uint32_t i = 0; i < n; ++i) {
        const V3<T> O = v3(T(O4[4 * i]), T(O4[4 * i + 1]), T(O4[4 * i + 2]));
        const V3<T> D = v3(T(D4[4 * i]), T(D4[4 * i + 1]), T(D4[4 * i + 2]));
        const V3<T> Tp = v3(T(T4[4 * i]), T(T4[4 * i + 1]), T(T4[4 * i + 2]));
        const T extendPdf = T(T4[4 * i + 3]);
        const uint32_t data = f2u(O4[4 * i + 3]);
        const uint32_t pathIx = data >> 4, flags = data & 15u;
        const uint32_t* h = hits + 4 * size_t(i);
        const T bu = decode16<T>(h[0] >> 16), bv = decode16<T>(h[0] & 0xFFFFu);
        const T tmax = T(u2f(h[3]));
        // hit record (bary, instIx, primIx within the instance's mesh, t) -> global triangle
        const uint32_t inst = h[2] == 0xffffffffu ? 0u : h[1];
        const uint32_t prim = (h[2] == 0xffffffffu || !s->twoLevel) ? h[2] : s->meshTriBase[s->instMesh[inst]] + h[2];
        ShadeOut<T> so;
        if (ref) {
            RefRng rng{tea2(st->seed + pathIx, sc + bounce + 1u)};
            so = shade_one<T, true>(*s, *st, bounce, O, D, Tp, extendPdf, pathIx, flags, prim, bu, bv, tmax, rng, inst);
        } else {
            CounterRng rng{pathIx % wh, sc + pathIx / wh, bounce + 1u, st->seed};
            so = shade_one<T, false>(*s, *st, bounce, O, D, Tp, extendPdf, pathIx, flags, prim, bu, bv, tmax, rng,
                                     inst);
        }
        ext_valid[i] = so.ext;
        sh_valid[i] = so.sh;
        float* e = ext + 12 * size_t(i);
        const float ev[12] = {float(so.extO.x), float(so.extO.y), float(so.extO.z), u2f(so.extPacked),
                              float(so.extD.x), float(so.extD.y), float(so.extD.z), u2f(so.extNormal),
                              float(so.extT.x), float(so.extT.y), float(so.extT.z), float(so.extPdf)};
        std::memcpy(e, ev, sizeof(ev));
        float* q = sh + 12 * size_t(i);
        const float sv[12] = {float(so.shO.x), float(so.shO.y), float(so.shO.z), u2f(pathIx),
                              float(so.shL.x), float(so.shL.y), float(so.shL.z), float(so.shDist),
                              float(so.shT.x), float(so.shT.y), float(so.shT.z), 0.f};
        std::memcpy(q, sv, sizeof(sv));
        radiance_add[4 * i] = float(so.add.x);
        radiance_add[4 * i + 1] = float(so.add.y);
        radiance_add[4 * i + 2] = float(so.add.z);
        radiance_add[4 * i + 3] = 0.f;
    }
}

} // namespace

extern "C" {

orc_scene* orc_scene_create(const tr_scene_desc* desc)
{
    if (!desc || (desc->instance_count ? !desc->meshes || !desc->instances : !desc->mesh))
        return nullptr;
    orc_scene* S = new orc_scene();
    S->twoLevel = desc->instance_count > 0;
    const uint32_t meshCount = S->twoLevel ? desc->mesh_count : 1u;
    auto meshOf = [&](uint32_t i) -> const tr_mesh_desc& { return S->twoLevel ? desc->meshes[i] : *desc->mesh; };
    uint32_t total = 0;
    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        S->meshTriBase.push_back(total);
        S->meshTriCount.push_back(meshOf(mi).triangle_count);
        total += meshOf(mi).triangle_count;
    }
    S->tris.resize(total);
    S->geo.resize(9 * size_t(total));
    S->geoD.resize(9 * size_t(total));
    S->matIdx.resize(total);
    for (uint32_t i = 0; i < desc->texture_count; ++i) {
        const tr_texture_desc& td = desc->textures[i];
        Texture t;
        t.w = td.width;
        t.h = td.height;
        t.texels.assign(td.texels, td.texels + 4 * size_t(td.width) * td.height);
        S->textures.push_back(std::move(t));
    }
    if (desc->material_textures && desc->texture_count > 0) {
        S->matTex.resize(size_t(desc->material_count) * TR_PROP_COUNT);
        for (size_t k = 0; k < S->matTex.size(); ++k) {
            const uint32_t ti = desc->material_textures[k];
            S->matTex[k] = ti == TR_NO_TEXTURE ? -1 : int32_t(ti);
        }
    }
    S->mats.resize(desc->material_count);
    for (uint32_t i = 0; i < desc->material_count; ++i) {
        const tr_material_desc& d = desc->materials[i];
        MatRaw& r = S->mats[i];
        for (int k = 0; k < 3; ++k) {
            r.diffuse[k] = hround(d.diffuse[k]);
            r.emissive[k] = hround(d.emissive[k]);
        }
        r.metallic = hround(d.metallic);
        r.subsurface = hround(d.subsurface);
        r.specular = hround(d.specular);
        r.roughness = hround(d.roughness);
        r.specularTint = hround(d.specular_tint);
        r.anisotropic = hround(d.anisotropic);
        r.sheen = hround(d.sheen);
        r.sheenTint = hround(d.sheen_tint);
        r.clearcoat = hround(d.clearcoat);
        r.clearcoatGloss = hround(d.clearcoat_gloss);
        r.closure = d.closure;
    }
    // Model::Build (Model.cpp:93-167), object space
    std::vector<V3<float>> lightN(total);
    for (uint32_t mi = 0; mi < meshCount; ++mi) {
        const tr_mesh_desc& m = meshOf(mi);
        const uint32_t base = S->meshTriBase[mi];
        const uint32_t offset = S->twoLevel && desc->mesh_material_offsets ? desc->mesh_material_offsets[mi] : 0u;
        for (uint32_t t = 0; t < m.triangle_count; ++t) {
            const uint32_t ix[3] = {m.indices[3 * t], m.indices[3 * t + 1], m.indices[3 * t + 2]};
            V3<float> p[3], nn[3];
            for (int k = 0; k < 3; ++k)
                p[k] = v3(m.positions[3 * ix[k]], m.positions[3 * ix[k] + 1], m.positions[3 * ix[k] + 2]);
            for (int k = 0; k < 3; ++k) {
                if (m.normals)
                    nn[k] = v3(m.normals[3 * ix[k]], m.normals[3 * ix[k] + 1], m.normals[3 * ix[k] + 2]);
                else
                    nn[k] = normalize(cross(p[1] - p[0], p[2] - p[0]));
            }
            Tri& tr = S->tris[base + t];
            for (int k = 0; k < 3; ++k) {
                tr.v[k][0] = p[k].x;
                tr.v[k][1] = p[k].y;
                tr.v[k][2] = p[k].z;
                tr.uv[k][0] = hbits(m.texcoords ? m.texcoords[2 * ix[k]] : 0.f);
                tr.uv[k][1] = hbits(m.texcoords ? m.texcoords[2 * ix[k] + 1] : 0.f);
                tr.n[k][0] = hbits(nn[k].x);
                tr.n[k][1] = hbits(nn[k].y);
                tr.n[k][2] = hbits(nn[k].z);
            }
            const V3<float> N = normalize(nn[0] + nn[1] + nn[2]);
            tr.N[0] = hbits(N.x);
            tr.N[1] = hbits(N.y);
            tr.N[2] = hbits(N.z);
            lightN[base + t] = normalize(normalize(nn[0] + nn[1] + nn[2]));
            float* g = &S->geo[9 * size_t(base + t)];
            double* gd = &S->geoD[9 * size_t(base + t)];
            for (int a = 0; a < 3; ++a) {
                g[a] = tr.v[0][a];
                g[3 + a] = tr.v[1][a] - tr.v[0][a];
                g[6 + a] = tr.v[2][a] - tr.v[0][a];
                gd[a] = double(tr.v[0][a]);
                gd[3 + a] = double(tr.v[1][a]) - double(tr.v[0][a]);
                gd[6 + a] = double(tr.v[2][a]) - double(tr.v[0][a]);
            }
            S->matIdx[base + t] = m.material_indices[t] + offset;
        }
    }
    // instances: inverse transforms (LinearMath.h:472-506), lights gathered in
    // instance then triangle order (Model::BuildLights, Model.cpp:205-230;
    // Scene::GatherLights, Scene.cpp:275-302): vertices placed with the instance
    // transform as the geometry is (R p + t), the normal with the inverse
    // transpose as the shading frame is, area in object space
    const uint32_t instCount = S->twoLevel ? desc->instance_count : 1u;
    std::vector<double> energies;
    float sumEnergy = 0.f;
    for (uint32_t i = 0; i < instCount; ++i) {
        const uint32_t mi = S->twoLevel ? desc->instances[i].mesh : 0u;
        S->instMesh.push_back(mi);
        float inv[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
        const float* xf = S->twoLevel ? desc->instances[i].transform : nullptr;
        if (xf) {
            const float xx = xf[0], xy = xf[1], xz = xf[2], tx = xf[3];
            const float yx = xf[4], yy = xf[5], yz = xf[6], ty = xf[7];
            const float zx = xf[8], zy = xf[9], zz = xf[10], tz = xf[11];
            const float det3 = xx * (yy * zz - yz * zy) - xy * (yx * zz - yz * zx) + xz * (yx * zy - yy * zx);
            const float id = 1.0f / det3;
            const float a00 = id * (yy * zz - zy * yz), a01 = id * (xz * zy - zz * xy), a02 = id * (xy * yz - yy * xz);
            const float a10 = id * (yz * zx - zz * yx), a11 = id * (xx * zz - zx * xz), a12 = id * (xz * yx - yz * xx);
            const float a20 = id * (yx * zy - zx * yy), a21 = id * (xy * zx - zy * xx), a22 = id * (xx * yy - yx * xy);
            const float r[12] = {a00, a01, a02, -a00 * tx - a01 * ty - a02 * tz,
                                 a10, a11, a12, -a10 * tx - a11 * ty - a12 * tz,
                                 a20, a21, a22, -a20 * tx - a21 * ty - a22 * tz};
            std::copy(r, r + 12, inv);
        }
        S->instInv.insert(S->instInv.end(), inv, inv + 12);
        const uint32_t base = S->meshTriBase[mi];
        for (uint32_t t = 0; t < S->meshTriCount[mi]; ++t) {
            const Tri& tr = S->tris[base + t];
            const tr_material_desc& md = desc->materials[S->matIdx[base + t]];
            const V3<float> em = v3(md.emissive[0], md.emissive[1], md.emissive[2]);
            if (!(em.x + em.y + em.z > kEps))
                continue;
            Light L{};
            L.triIx = base + t;
            V3<float> p[3];
            for (int k = 0; k < 3; ++k)
                p[k] = v3(tr.v[k][0], tr.v[k][1], tr.v[k][2]);
            float* dst[3] = {L.V0, L.V1, L.V2};
            for (int k = 0; k < 3; ++k) {
                V3<float> w = p[k];
                if (xf)
                    w = v3(((xf[0] * p[k].x + xf[1] * p[k].y) + xf[2] * p[k].z) + xf[3],
                           ((xf[4] * p[k].x + xf[5] * p[k].y) + xf[6] * p[k].z) + xf[7],
                           ((xf[8] * p[k].x + xf[9] * p[k].y) + xf[10] * p[k].z) + xf[11]);
                dst[k][0] = w.x;
                dst[k][1] = w.y;
                dst[k][2] = w.z;
            }
            V3<float> ln = lightN[base + t];
            if (xf) {
                const V3<float> n0 = ln;
                ln = normalize(v3((n0.x * inv[0] + n0.y * inv[4]) + n0.z * inv[8],
                                  (n0.x * inv[1] + n0.y * inv[5]) + n0.z * inv[9],
                                  (n0.x * inv[2] + n0.y * inv[6]) + n0.z * inv[10]));
                ln = normalize(ln);
            }
            L.N[0] = ln.x;
            L.N[1] = ln.y;
            L.N[2] = ln.z;
            const float a = length(p[1] - p[0]), b = length(p[2] - p[1]), c = length(p[0] - p[2]);
            const float sp = (a + b + c) * .5f;
            L.area = msqrt(sp * (sp - a) * (sp - b) * (sp - c));
            L.radiance[0] = em.x;
            L.radiance[1] = em.y;
            L.radiance[2] = em.z;
            const V3<float> e = em * L.area;
            L.energy = e.x + e.y + e.z;
            L.sumEnergy = sumEnergy;
            sumEnergy += L.energy;
            S->lights.push_back(L);
            energies.push_back(double(L.energy));
        }
    }
    S->lightEnergy = S->lights.empty() ? 0.f : S->lights.back().sumEnergy;
    S->lightEnergyTotal = sumEnergy;
    S->alias = alias_table(energies);
    build_bvh(*S);
    return S;
}

void orc_scene_destroy(orc_scene* s) { delete s; }

void orc_texture_sample(const orc_scene* s, uint32_t texture, float u, float v, float* out)
{
    texture_sample(s->textures[texture], u, v, out);
}

// Sky::SetSunDir (normalised with helper_math's normalize), SetTurbidity (clamp to
// [1, 10]) and Sky::Build (cos of the angular diameter in radians); NULL disables.
void orc_set_sky(orc_scene* s, const tr_sky_desc* sky)
{
    if (!sky) {
        s->sky.enabled = 0;
        return;
    }
    const float* d = sky->sun_dir;
    const float inv = 1.0f / std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    for (int i = 0; i < 3; ++i)
        s->sky.sunDir[i] = d[i] * inv;
    s->sky.enabled = sky->enabled ? 1 : 0;
    s->sky.drawSun = sky->draw_sun ? 1.f : 0.f;
    s->sky.cosSunAngularDiameter = std::cos(sky->sun_angular_diameter * K<float>::Pi / (60.f * 180.f));
    s->sky.sunIntensity = sky->sun_intensity;
    s->sky.turbidity = std::fmin(std::fmax(sky->turbidity, 1.f), 10.f);
}
uint32_t orc_light_count(const orc_scene* s) { return uint32_t(s->lights.size()); }
float orc_light_energy(const orc_scene* s, int total) { return total ? s->lightEnergyTotal : s->lightEnergy; }

void orc_generate(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                  uint32_t sc, uint32_t first, uint32_t n, float* O4, float* D4, float* T4)
{
    (void)s;
    const uint32_t wh = W * H;
    const float tanFov2 = std::tan(cam->fov / 2.0f);
    const bool ref = st->flags & TR_FLAG_REFERENCE_SAMPLING;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t pathIx = first + k;
        const uint32_t pixel = pathIx % wh;
        V3<float> O, D;
        float Tv;
        if (ref) {
            RefRng rng{tea2(st->seed + pathIx, sc << 1)};
            camera_ray<float>(*cam, tanFov2, W, H, pixel % W, pixel / W, rng, O, D, Tv);
        } else {
            CounterRng rng{pixel, sc + pathIx / wh, 0u, st->seed};
            camera_ray<float>(*cam, tanFov2, W, H, pixel % W, pixel / W, rng, O, D, Tv);
        }
        const float o[4] = {O.x, O.y, O.z, u2f(pathIx << 4)};
        const float d[4] = {D.x, D.y, D.z, 0.f};
        const float t[4] = {Tv, Tv, Tv, 1.f};
        std::memcpy(O4 + 4 * size_t(k), o, 16);
        std::memcpy(D4 + 4 * size_t(k), d, 16);
        std::memcpy(T4 + 4 * size_t(k), t, 16);
    }
}

// RayPick raygen, optix.cu:345-377 (DeviceRenderer::PickRay, DeviceRenderer.cpp:71-92): the
// camera ray of pixel (x, H - y) with the LCG state 0, closest hit; out = RayPickResult words.
void orc_pick_ray(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
                  int32_t x, int32_t y, float* out)
{
    const float tanFov2 = std::tan(cam->fov / 2.0f);
    RefRng rng{0u};
    V3<float> O, D;
    float Tv;
    camera_ray<float>(*cam, tanFov2, W, H, x, int(H) - y, rng, O, D, Tv);
    uint32_t inst = 0xffffffffu, prim = 0xffffffffu;
    float tmax = kDstMax;
    if (Tv > 0) {
        const float Oa[3] = {O.x, O.y, O.z}, Da[3] = {D.x, D.y, D.z};
        float t = kDstMax, u = 0, v = 0;
        uint32_t p = 0xffffffffu, in = 0;
        if (trace<float>(*s, Oa, Da, st->ray_epsilon, t, false, p, u, v, &in)) {
            inst = in;
            prim = s->twoLevel ? p - s->meshTriBase[s->instMesh[in]] : p;
            tmax = t;
        }
    }
    const float r[9] = {cam->position[0], cam->position[1], cam->position[2], u2f(inst), D.x, D.y, D.z, u2f(prim),
                        tmax};
    std::memcpy(out, r, sizeof(r));
}

void orc_trace_closest(const orc_scene* s, const float* O4, const float* D4, uint32_t n, float tmin, uint32_t* hits)
{
    for (uint32_t i = 0; i < n; ++i) {
        const float O[3] = {O4[4 * i], O4[4 * i + 1], O4[4 * i + 2]};
        const float D[3] = {D4[4 * i], D4[4 * i + 1], D4[4 * i + 2]};
        float tmax = kDstMax, u = 0, v = 0;
        uint32_t prim = 0xffffffffu, inst = 0;
        uint32_t* h = hits + 4 * size_t(i);
        if (trace<float>(*s, O, D, tmin, tmax, false, prim, u, v, &inst)) {
            h[0] = encode_bary(u, v);
            h[1] = inst;
            h[2] = s->twoLevel ? prim - s->meshTriBase[s->instMesh[inst]] : prim;
            h[3] = f2u(tmax);
        } else {
            h[0] = 0;
            h[1] = 0xffffffffu;
            h[2] = 0xffffffffu;
            h[3] = f2u(kDstMax);
        }
    }
}

int orc_trace_ray(const orc_scene* s, const float* O, const float* D, float tmin, float tmax, int any, uint32_t* prim,
                  float* t, float* u, float* v, uint32_t* inst)
{
    float tm = tmax, uu = 0, vv = 0;
    uint32_t p = 0xffffffffu, in = 0;
    if (!trace<float>(*s, O, D, tmin, tm, any != 0, p, uu, vv, &in))
        return 0;
    *prim = s->twoLevel ? p - s->meshTriBase[s->instMesh[in]] : p;
    if (inst)
        *inst = in;
    *t = tm;
    *u = uu;
    *v = vv;
    return 1;
}

uint32_t orc_ties(const orc_scene* s, const float* O, const float* D, float tmin, float t, float rel, uint32_t* prims,
                  uint32_t max_out, uint32_t* insts)
{
    uint32_t count = 0;
    const uint32_t instCount = s->twoLevel ? uint32_t(s->instMesh.size()) : 1u;
    for (uint32_t i = 0; i < instCount; ++i) {
        float Oo[3] = {O[0], O[1], O[2]}, Do[3] = {D[0], D[1], D[2]};
        uint32_t base = 0, end = uint32_t(s->tris.size());
        if (s->twoLevel) {
            to_object<float>(&s->instInv[12 * size_t(i)], O, D, Oo, Do);
            base = s->meshTriBase[s->instMesh[i]];
            end = base + s->meshTriCount[s->instMesh[i]];
        }
        for (uint32_t p = base; p < end; ++p) {
            float tt, u, v;
            if (tri_test_f(&s->geo[9 * size_t(p)], Oo, Do, tmin, kDstMax, tt, u, v) &&
                mfabs(tt - t) <= rel * mfabs(t)) {
                if (count < max_out) {
                    prims[count] = p - base;
                    if (insts)
                        insts[count] = i;
                }
                ++count;
            }
        }
    }
    return count;
}

void orc_trace_any(const orc_scene* s, const float* O4, const float* L4, uint32_t n, float eps, uint8_t* occluded)
{
    for (uint32_t i = 0; i < n; ++i) {
        const float O[3] = {O4[4 * i], O4[4 * i + 1], O4[4 * i + 2]};
        const float D[3] = {L4[4 * i], L4[4 * i + 1], L4[4 * i + 2]};
        float tmax = L4[4 * i + 3] - (2 * eps);
        uint32_t prim = 0;
        float u, v;
        occluded[i] = trace<float>(*s, O, D, eps, tmax, true, prim, u, v) ? 1 : 0;
    }
}

void orc_shade(const orc_scene* s, const tr_kernel_settings* st, uint32_t bounce, uint32_t sc, uint32_t W, uint32_t H,
               uint32_t n, const float* O4, const float* D4, const float* T4, const uint32_t* hits, float* ext,
               uint8_t* ext_valid, float* sh, uint8_t* sh_valid, float* radiance_add)
{
    shade_entries<float>(s, st, bounce, sc, W, H, n, O4, D4, T4, hits, ext, ext_valid, sh, sh_valid, radiance_add);
}

void orc_shade_fp64(const orc_scene* s, const tr_kernel_settings* st, uint32_t bounce, uint32_t sc, uint32_t W,
                    uint32_t H, uint32_t n, const float* O4, const float* D4, const float* T4, const uint32_t* hits,
                    float* ext, uint8_t* ext_valid, float* sh, uint8_t* sh_valid, float* radiance_add)
{
    shade_entries<double>(s, st, bounce, sc, W, H, n, O4, D4, T4, hits, ext, ext_valid, sh, sh_valid, radiance_add);
}

int orc_render(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t W, uint32_t H,
               uint32_t frames, uint32_t first_pixel, uint32_t pixel_count, int use_double, int threads,
               double* accumulator, double* path_radiance, uint64_t* ray_counts)
{
    const uint32_t wh = W * H;
    const uint32_t ms = st->multi_sample;
    const bool ref = st->flags & TR_FLAG_REFERENCE_SAMPLING;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = threads > 0 ? unsigned(threads) : hw;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> totExt{0}, totSh{0};
    const float tanFov2f = std::tan(cam->fov / 2.0f);
    auto worker = [&]() {
        uint64_t nExt = 0, nSh = 0;
        while (true) {
            const uint32_t chunk = next.fetch_add(64);
            if (chunk >= pixel_count)
                break;
            const uint32_t end = std::min(pixel_count, chunk + 64);
            for (uint32_t k = chunk; k < end; ++k) {
                const uint32_t pixel = first_pixel + k;
                double acc[3] = {0, 0, 0};
                for (uint32_t f = 0; f < frames; ++f) {
                    const uint32_t sc = f * ms;
                    double frameSum[3] = {0, 0, 0};
                    for (uint32_t smp = 0; smp < ms; ++smp) {
                        const uint32_t pathIx = pixel + smp * wh;
                        double r[3];
                        if (use_double) {
                            const V3<double> v =
                                ref ? render_path<double, true>(*s, *cam, double(tanFov2f), *st, W, H, sc, pathIx, nExt, nSh)
                                    : render_path<double, false>(*s, *cam, double(tanFov2f), *st, W, H, sc, pathIx, nExt, nSh);
                            r[0] = v.x; r[1] = v.y; r[2] = v.z;
                        } else {
                            const V3<float> v =
                                ref ? render_path<float, true>(*s, *cam, tanFov2f, *st, W, H, sc, pathIx, nExt, nSh)
                                    : render_path<float, false>(*s, *cam, tanFov2f, *st, W, H, sc, pathIx, nExt, nSh);
                            r[0] = v.x; r[1] = v.y; r[2] = v.z;
                        }
                        if (path_radiance && f + 1 == frames) {
                            double* pr = path_radiance + 4 * (size_t(smp) * pixel_count + k);
                            pr[0] = r[0]; pr[1] = r[1]; pr[2] = r[2]; pr[3] = 0.0;
                        }
                        for (int c = 0; c < 3; ++c)
                            frameSum[c] += r[c];
                    }
                    for (int c = 0; c < 3; ++c)
                        acc[c] += frameSum[c];
                }
                double* a = accumulator + 4 * size_t(k);
                a[0] = acc[0]; a[1] = acc[1]; a[2] = acc[2];
                a[3] = double(frames) * double(ms);
            }
        }
        totExt += nExt;
        totSh += nSh;
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t)
        pool.emplace_back(worker);
    worker();
    for (auto& t : pool)
        t.join();
    if (ray_counts) {
        ray_counts[0] += totExt.load();
        ray_counts[1] += totSh.load();
    }
    return 0;
}

void orc_counter_rng(uint32_t pixel, uint32_t sample, uint32_t bounce, uint32_t seed, uint32_t n, float* out)
{
    CounterRng r{pixel, sample, bounce, seed};
    for (uint32_t i = 0; i < n; ++i)
        out[i] = r.next();
}

void orc_closure(int type, int reference, int use_double, const float* in, float* out)
{
    auto run = [&](auto zero) {
        using T = decltype(zero);
        const V3<T> wo = v3(T(in[0]), T(in[1]), T(in[2]));
        const V3<T> wi = v3(T(in[3]), T(in[4]), T(in[5]));
        const V3<T> Tp = v3(T(in[6]), T(in[7]), T(in[8]));
        const float* q = in + 9;
        HitMat<T> m;
        m.diffuse = v3(T(q[0]), T(q[1]), T(q[2]));
        m.metallic = T(q[3]);
        m.emissive = v3(T(q[4]), T(q[5]), T(q[6]));
        m.subsurface = T(q[7]);
        m.tint = v3(T(q[8]), T(q[9]), T(q[10]));
        m.specular = T(q[11]);
        m.roughness = T(q[12]);
        m.specularTint = T(q[13]);
        m.anisotropic = T(q[14]);
        m.sheen = T(q[15]);
        m.sheenTint = T(q[16]);
        m.clearcoat = T(q[17]);
        m.clearcoatGloss = T(q[18]);
        m.luminance = T(q[19]);
        m.closure = uint32_t(type);
        const T r0 = T(q[20]), r1 = T(q[21]);
        Clos<T> c;
        if (type == TR_CLOSURE_DISNEY)
            c = reference ? finalize(Tp, d_evaluate<T, true>(wo, wi, m), d_sample<T, true>(wo, m, r0, r1))
                          : d_closure_default<T>(wo, wi, Tp, m, r0, r1);
        else if (type == TR_CLOSURE_DIFFUSE)
            c = diffuse(wo, wi, Tp, m, r0, r1);
        else
            c = lambert(wo, wi, Tp, m, r0, r1);
        const float o[14] = {float(c.extT.x), float(c.extT.y), float(c.extT.z), float(c.extPdf),
                             float(c.extWi.x), float(c.extWi.y), float(c.extWi.z), u2f(c.extFlags),
                             float(c.shT.x), float(c.shT.y), float(c.shT.z), float(c.shPdf), 0.f, 0.f};
        std::memcpy(out, o, sizeof(o));
    };
    if (use_double)
        run(0.0);
    else
        run(0.0f);
}

int orc_adjoint(const orc_scene* s, const tr_camera* cam, const tr_kernel_settings* st, uint32_t width,
                uint32_t height, uint32_t sample_count, const float* pixel_grad, float scale, int use_double,
                int threads, double* grads)
{
    if (st->flags & TR_FLAG_REFERENCE_SAMPLING)
        return 1;
    const uint32_t wh = width * height;
    const uint32_t n = wh * st->multi_sample;
    const size_t m = s->mats.size() * 9;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = threads > 0 ? unsigned(threads) : hw;
    std::vector<std::vector<double>> partial(nt, std::vector<double>(m, 0.0));
    std::atomic<uint32_t> next{0};
    const float tanFov2f = std::tan(cam->fov / 2.0f);
    auto worker = [&](unsigned t) {
        while (true) {
            const uint32_t chunk = next.fetch_add(256);
            if (chunk >= n)
                break;
            for (uint32_t p = chunk; p < std::min(n, chunk + 256); ++p) {
                const uint32_t px = p % wh;
                const double delta[3] = {double(pixel_grad[4 * px]) * scale, double(pixel_grad[4 * px + 1]) * scale,
                                         double(pixel_grad[4 * px + 2]) * scale};
                if (delta[0] == 0 && delta[1] == 0 && delta[2] == 0)
                    continue;
                if (use_double)
                    adjoint_path<double>(*s, *cam, double(tanFov2f), *st, width, height, sample_count, p, delta,
                                         partial[t].data());
                else
                    adjoint_path<float>(*s, *cam, tanFov2f, *st, width, height, sample_count, p, delta,
                                        partial[t].data());
            }
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t)
        pool.emplace_back(worker, t);
    worker(0);
    for (auto& th : pool)
        th.join();
    for (size_t k = 0; k < m; ++k) {
        double acc = 0.0;
        for (unsigned t = 0; t < nt; ++t)
            acc += partial[t][k];
        grads[k] += acc;
    }
    return 0;
}

void orc_closure_value_grad(const orc_scene* s, uint32_t material, const float* wo, const float* wi, double* out)
{
    const V3<double> o = v3(double(wo[0]), double(wo[1]), double(wo[2]));
    const V3<double> i = v3(double(wi[0]), double(wi[1]), double(wi[2]));
    const V3<DualT<double>> f = dual_value<double>(*s, material, o, i);
    const DualT<double>* fc[3] = {&f.x, &f.y, &f.z};
    for (int c = 0; c < 3; ++c) {
        out[7 * c] = fc[c]->v;
        for (int p = 0; p < kDP; ++p)
            out[7 * c + 1 + p] = fc[c]->d[p];
    }
}

void orc_set_reference_draw_order(int right_to_left) { g_refRightToLeft = right_to_left != 0; }

void orc_reference_rng(uint32_t v0, uint32_t v1, uint32_t n, float* out)
{
    RefRng r{tea2(v0, v1)};
    for (uint32_t i = 0; i < n; ++i)
        out[i] = r.next();
}

} // extern "C"

// Scene files: the reference's scene JSON (Tracer/FileIO/SceneFile.cpp), its
// model and texture cache formats (ModelFile.cpp / TextureFile.cpp over
// BinaryFile.h/.inl) and Wavefront OBJ, read into a two-level tr_scene_desc.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "../../include/trayracer.h"
#include "tr_json.h"

namespace tr {
namespace {

thread_local std::string g_error;

tr_status sf_fail(tr_status st, const std::string& msg)
{
    g_error = msg;
    return st;
}

constexpr float kDegToRad = 3.14159265359f / 180.f;  // LinearMath.h:41

// ------------------------------------------------------------------ paths

bool is_absolute(const std::string& p) { return !p.empty() && p[0] == '/'; }

std::string join(const std::string& dir, const std::string& p)
{
    if (is_absolute(p) || dir.empty())
        return p;
    return dir.back() == '/' ? dir + p : dir + "/" + p;
}

std::string directory_of(const std::string& p)
{
    const size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : (k == 0 ? std::string("/") : p.substr(0, k));
}

std::string current_dir()
{
    char buf[4096];
    return getcwd(buf, sizeof(buf)) ? std::string(buf) : std::string(".");
}

bool read_file(const std::string& path, std::vector<char>& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    if (n < 0)
        return false;
    f.seekg(0, std::ios::beg);
    out.resize(size_t(n));
    if (n > 0)
        f.read(out.data(), n);
    return bool(f) || n == 0;
}

bool file_time(const std::string& path, int64_t& t)
{
    struct stat st;
    if (stat(path.c_str(), &st) != 0)
        return false;
    t = int64_t(st.st_mtime);
    return true;
}

std::string lower(std::string s)
{
    for (char& c : s)
        if (c >= 'A' && c <= 'Z')
            c = char(c - 'A' + 'a');
    return s;
}

// BinaryFile::CachedFilePath (BinaryFile.cpp:67-71): "cache/" + std::hash of the
// path + ".bin". The reference is built with MSVC, whose std::hash of a string
// is 64-bit FNV-1a over its bytes (Fowler, Noll, Vo).
uint64_t fnv1a64(const std::string& s)
{
    uint64_t h = 14695981039346656037ull;
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
    return h;
}

std::string cache_path(const std::string& base, const std::string& globalPath)
{
    return join(base, "cache/" + std::to_string(fnv1a64(globalPath)) + ".bin");
}

// ------------------------------------------------------------------ BinaryFile format
// Little-endian raw values; strings and vectors carry a 64-bit element count
// first (BinaryFile.inl); the header is three type characters and a version byte.
struct Reader {
    const std::vector<char>& buf;
    size_t head = 0;
    bool ok = true;

    explicit Reader(const std::vector<char>& b) : buf(b) {}

    bool raw(void* dst, size_t n)
    {
        if (!ok || n > buf.size() - head) {
            ok = false;
            return false;
        }
        if (n)
            std::memcpy(dst, buf.data() + head, n);
        head += n;
        return true;
    }
    template <class T> bool value(T& v) { return raw(&v, sizeof(T)); }
    bool count(uint64_t& n, size_t elem)
    {
        if (!value(n))
            return false;
        if (elem && n > (buf.size() - head) / elem) {
            ok = false;
            return false;
        }
        return true;
    }
    bool string(std::string& s)
    {
        uint64_t n;
        if (!count(n, 1))
            return false;
        s.assign(buf.data() + head, size_t(n));
        head += size_t(n);
        return true;
    }
    template <class T> bool vec(std::vector<T>& v, size_t comps)
    {
        uint64_t n;
        if (!count(n, sizeof(T) * comps))
            return false;
        v.resize(size_t(n) * comps);
        return raw(v.data(), v.size() * sizeof(T));
    }
};

struct Writer {
    std::vector<char> buf;
    void raw(const void* src, size_t n)
    {
        const size_t o = buf.size();
        buf.resize(o + n);
        if (n)
            std::memcpy(buf.data() + o, src, n);
    }
    template <class T> void value(const T& v) { raw(&v, sizeof(T)); }
    void string(const std::string& s)
    {
        value(uint64_t(s.size()));
        raw(s.data(), s.size());
    }
    template <class T> void vec(const T* p, size_t elems, size_t comps)
    {
        value(uint64_t(elems));
        raw(p, elems * comps * sizeof(T));
    }
    bool save(const std::string& path) const
    {
        std::ofstream f(path, std::ios::binary | std::ios::trunc);
        if (!f)
            return false;
        f.write(buf.data(), std::streamsize(buf.size()));
        return bool(f);
    }
};

bool header_is(const std::vector<char>& b, const char id[3], uint8_t version)
{
    return b.size() >= 4 && b[0] == id[0] && b[1] == id[1] && b[2] == id[2] && uint8_t(b[3]) == version;
}

const char kModelId[3] = {'M', 'D', 'L'};
const char kTextureId[3] = {'T', 'E', 'X'};
constexpr uint8_t kCacheVersion = 2;

// ------------------------------------------------------------------ materials
// Material::Material (Material.cpp:98-112): the 13 properties in
// MaterialPropertyIds order, each a float colour, an RGB colour and/or a texture.
enum PropKind : uint32_t { kFloat = 1, kRgb = 2, kTex = 4 };
constexpr uint32_t kPropKinds[TR_PROP_COUNT] = {
    kFloat | kTex,  // Anisotropic
    kFloat | kTex,  // Clearcoat
    kFloat | kTex,  // ClearcoatGloss
    kRgb | kTex,    // Diffuse
    kRgb,           // Emissive
    kFloat | kTex,  // Metallic
    kTex,           // Normal
    kFloat | kTex,  // Roughness
    kFloat | kTex,  // Sheen
    kFloat | kTex,  // SheenTint
    kFloat | kTex,  // Specular
    kFloat | kTex,  // SpecularTint
    kFloat | kTex,  // Subsurface
};
const char* const kPropNames[TR_PROP_COUNT] = {"anisotropic", "clearcoat", "clearcoatgloss", "diffuse",
                                               "emissive", "metallic", "normal", "roughness", "sheen",
                                               "sheentint", "specular", "speculartint", "subsurface"};

// a material as the reference holds it: each property's colour (x only for
// float properties) and texture path
struct MaterialRec {
    std::string name;
    float color[TR_PROP_COUNT][3] = {};
    std::string tex[TR_PROP_COUNT];

    MaterialRec()
    {
        for (auto& c : color)
            c[0] = c[1] = c[2] = 0.f;
        for (int k = 0; k < 3; ++k)
            color[TR_PROP_DIFFUSE][k] = 1.f;
        color[TR_PROP_ROUGHNESS][0] = 1.f;
    }
};

float* desc_scalar(tr_material_desc& d, uint32_t p)
{
    switch (p) {
    case TR_PROP_ANISOTROPIC: return &d.anisotropic;
    case TR_PROP_CLEARCOAT: return &d.clearcoat;
    case TR_PROP_CLEARCOAT_GLOSS: return &d.clearcoat_gloss;
    case TR_PROP_METALLIC: return &d.metallic;
    case TR_PROP_ROUGHNESS: return &d.roughness;
    case TR_PROP_SHEEN: return &d.sheen;
    case TR_PROP_SHEEN_TINT: return &d.sheen_tint;
    case TR_PROP_SPECULAR: return &d.specular;
    case TR_PROP_SPECULAR_TINT: return &d.specular_tint;
    case TR_PROP_SUBSURFACE: return &d.subsurface;
    default: return nullptr;
    }
}

tr_material_desc to_desc(const MaterialRec& m)
{
    tr_material_desc d{};
    for (int k = 0; k < 3; ++k) {
        d.diffuse[k] = m.color[TR_PROP_DIFFUSE][k];
        d.emissive[k] = m.color[TR_PROP_EMISSIVE][k];
    }
    for (uint32_t p = 0; p < TR_PROP_COUNT; ++p)
        if (float* f = desc_scalar(d, p))
            *f = m.color[p][0];
    d.closure = TR_CLOSURE_LAMBERT;
    return d;
}

MaterialRec from_desc(const tr_material_desc& d, const char* name)
{
    MaterialRec m;
    m.name = name ? name : "";
    for (int k = 0; k < 3; ++k) {
        m.color[TR_PROP_DIFFUSE][k] = d.diffuse[k];
        m.color[TR_PROP_EMISSIVE][k] = d.emissive[k];
    }
    tr_material_desc c = d;
    for (uint32_t p = 0; p < TR_PROP_COUNT; ++p)
        if (float* f = desc_scalar(c, p))
            m.color[p][0] = *f;
    return m;
}

// ------------------------------------------------------------------ models
struct ModelData {
    std::string name;
    std::vector<float> pos, nrm, uv;   // 3, 3, 2 floats per vertex
    std::vector<uint32_t> idx, matIdx; // 3 per triangle, 1 per triangle
    std::vector<MaterialRec> mats;
};

// LoadFromCache (ModelFile.cpp:98-160): header, vertices, normals, texcoords,
// indices, material indices, then the materials with their property values and
// texture paths in MaterialPropertyIds order.
bool read_model_cache(const std::vector<char>& buf, ModelData& m, std::string& err)
{
    if (!header_is(buf, kModelId, kCacheVersion)) {
        err = "not a model cache file (MDL version 2)";
        return false;
    }
    Reader r(buf);
    r.head = 4;
    r.vec(m.pos, 3);
    r.vec(m.nrm, 3);
    r.vec(m.uv, 2);
    r.vec(m.idx, 3);
    r.vec(m.matIdx, 1);
    uint64_t matCount = 0;
    r.count(matCount, 8);
    for (uint64_t i = 0; i < matCount && r.ok; ++i) {
        MaterialRec mat;
        r.string(mat.name);
        for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
            if (kPropKinds[p] & kFloat)
                r.value(mat.color[p][0]);
            if (kPropKinds[p] & kRgb)
                r.raw(mat.color[p], 3 * sizeof(float));
            if (kPropKinds[p] & kTex)
                r.string(mat.tex[p]);
        }
        m.mats.push_back(std::move(mat));
    }
    if (!r.ok) {
        err = "truncated model cache file";
        return false;
    }
    const size_t nv = m.pos.size() / 3;
    if (m.nrm.size() != m.pos.size() || m.uv.size() != 2 * nv || m.matIdx.size() != m.idx.size() / 3) {
        err = "model cache arrays disagree in length";
        return false;
    }
    return true;
}

void write_model_cache(Writer& w, const ModelData& m)
{
    const char hdr[4] = {kModelId[0], kModelId[1], kModelId[2], char(kCacheVersion)};
    w.raw(hdr, 4);
    w.vec(m.pos.data(), m.pos.size() / 3, 3);
    w.vec(m.nrm.data(), m.nrm.size() / 3, 3);
    w.vec(m.uv.data(), m.uv.size() / 2, 2);
    w.vec(m.idx.data(), m.idx.size() / 3, 3);
    w.vec(m.matIdx.data(), m.matIdx.size(), 1);
    w.value(uint64_t(m.mats.size()));
    for (const MaterialRec& mat : m.mats) {
        w.string(mat.name);
        for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
            if (kPropKinds[p] & kFloat)
                w.value(mat.color[p][0]);
            if (kPropKinds[p] & kRgb)
                w.raw(mat.color[p], 3 * sizeof(float));
            if (kPropKinds[p] & kTex)
                w.string(mat.tex[p]);
        }
    }
}

struct TextureData {
    uint32_t w = 0, h = 0;
    std::vector<uint16_t> texels;   // RGBA binary16
};

// Texture LoadFromCache (TextureFile.cpp:52-80): header, int2 resolution, half4 pixels.
bool read_texture_cache(const std::vector<char>& buf, TextureData& t, std::string& err)
{
    if (!header_is(buf, kTextureId, kCacheVersion)) {
        err = "not a texture cache file (TEX version 2)";
        return false;
    }
    Reader r(buf);
    r.head = 4;
    int32_t res[2] = {0, 0};
    r.raw(res, sizeof(res));
    r.vec(t.texels, 4);
    if (!r.ok || res[0] <= 0 || res[1] <= 0 || t.texels.size() != 4 * size_t(res[0]) * size_t(res[1])) {
        err = "malformed texture cache file";
        return false;
    }
    t.w = uint32_t(res[0]);
    t.h = uint32_t(res[1]);
    return true;
}

// Vertex normals as the normalised sum of the unit normals of the faces around
// each vertex's position (posOf: position index of each vertex; positions
// shared by several vertices share the sum).
void smooth_normals(const std::vector<float>& pos, const std::vector<uint32_t>& idx, const std::vector<int64_t>& posOf,
                    size_t positions, std::vector<float>& out)
{
    std::vector<float> acc(3 * positions, 0.f);
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const float* a = &pos[3 * size_t(idx[t])];
        const float* b = &pos[3 * size_t(idx[t + 1])];
        const float* c = &pos[3 * size_t(idx[t + 2])];
        const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const float e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const float n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                            e1[0] * e2[1] - e1[1] * e2[0]};
        const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (!(l > 0.f))
            continue;
        for (int k = 0; k < 3; ++k)
            for (int q = 0; q < 3; ++q)
                acc[3 * size_t(posOf[idx[t + size_t(k)]]) + size_t(q)] += n[q] / l;
    }
    out.assign(3 * posOf.size(), 0.f);
    for (size_t v = 0; v < posOf.size(); ++v) {
        const float* a = &acc[3 * size_t(posOf[v])];
        const float l = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        for (int q = 0; q < 3; ++q)
            out[3 * v + size_t(q)] = l > 0.f ? a[q] / l : (q == 1 ? 1.f : 0.f);
    }
}

// ------------------------------------------------------------------ Wavefront OBJ
// Stands in for the reference's Assimp import of OBJ models (ModelFile.cpp:
// 331-449): polygons become triangle fans, each distinct (position, texcoord,
// normal) triple one vertex; vertices without a normal take the normalised sum
// of the unit normals of the faces around their position. Materials come from
// the mtllib files: Kd, Ke, map_Kd (diffuse), map_Ks (specular), norm / map_Bump /
// bump (normal), map_Pm (metallic) and map_Pr (roughness), as the reference
// takes them from Assimp.
bool read_obj(const std::string& path, ModelData& m, std::string& err)
{
    std::ifstream f(path);
    if (!f) {
        err = "cannot open " + path;
        return false;
    }
    const std::string dir = directory_of(path);
    std::vector<float> P, T, N;
    std::map<std::array<int64_t, 3>, uint32_t> vmap;
    std::map<std::string, uint32_t> matIndex;
    std::vector<int64_t> vertPos;   // position index per output vertex
    std::vector<bool> hasNormal;
    uint32_t curMat = 0;
    bool anyMat = false;
    auto material_named = [&](const std::string& name) {
        auto it = matIndex.find(name);
        if (it != matIndex.end())
            return it->second;
        MaterialRec r;
        r.name = name;
        m.mats.push_back(r);
        return matIndex[name] = uint32_t(m.mats.size() - 1);
    };
    auto read_mtl = [&](const std::string& file) {
        std::ifstream mf(join(dir, file));
        std::string line;
        MaterialRec* cur = nullptr;
        while (std::getline(mf, line)) {
            std::istringstream ls(line);
            std::string k;
            ls >> k;
            if (k == "newmtl") {
                std::string name;
                std::getline(ls >> std::ws, name);
                cur = &m.mats[material_named(name)];
            } else if (cur && (k == "Kd" || k == "Ke")) {
                float c[3] = {0, 0, 0};
                ls >> c[0] >> c[1] >> c[2];
                float* dst = cur->color[k == "Kd" ? TR_PROP_DIFFUSE : TR_PROP_EMISSIVE];
                std::copy(c, c + 3, dst);
            } else if (cur) {
                const std::pair<const char*, uint32_t> maps[] = {
                    {"map_kd", TR_PROP_DIFFUSE}, {"map_ks", TR_PROP_SPECULAR}, {"norm", TR_PROP_NORMAL},
                    {"map_bump", TR_PROP_NORMAL}, {"bump", TR_PROP_NORMAL}, {"map_pm", TR_PROP_METALLIC},
                    {"map_pr", TR_PROP_ROUGHNESS}};
                for (const auto& mp : maps)
                    if (lower(k) == mp.first) {
                        std::string name;
                        std::getline(ls >> std::ws, name);
                        // the texture path is the last token (options come first)
                        const size_t sp = name.find_last_of(" \t");
                        cur->tex[mp.second] = join(dir, sp == std::string::npos ? name : name.substr(sp + 1));
                    }
            }
        }
    };
    std::string line;
    size_t lineNo = 0;
    while (std::getline(f, line)) {
        ++lineNo;
        std::istringstream ls(line);
        std::string k;
        ls >> k;
        if (k == "v" || k == "vn") {
            float x = 0, y = 0, z = 0;
            ls >> x >> y >> z;
            auto& dst = k == "v" ? P : N;
            dst.insert(dst.end(), {x, y, z});
        } else if (k == "vt") {
            float x = 0, y = 0;
            ls >> x >> y;
            T.insert(T.end(), {x, y});
        } else if (k == "mtllib") {
            std::string file;
            while (ls >> file)
                read_mtl(file);
        } else if (k == "usemtl") {
            std::string name;
            std::getline(ls >> std::ws, name);
            curMat = material_named(name);
            anyMat = true;
        } else if (k == "f") {
            std::vector<uint32_t> face;
            std::string tok;
            while (ls >> tok) {
                int64_t ix[3] = {0, 0, 0};
                int slot = 0;
                std::string num;
                for (size_t c = 0; c <= tok.size(); ++c) {
                    if (c == tok.size() || tok[c] == '/') {
                        if (slot < 3 && !num.empty())
                            ix[slot] = std::stoll(num);
                        num.clear();
                        ++slot;
                    } else {
                        num += tok[c];
                    }
                }
                // 1-based, negative counts from the end
                const int64_t counts[3] = {int64_t(P.size() / 3), int64_t(T.size() / 2), int64_t(N.size() / 3)};
                for (int q = 0; q < 3; ++q) {
                    if (ix[q] < 0)
                        ix[q] = counts[q] + ix[q] + 1;
                    if (ix[q] < 0 || ix[q] > counts[q] || (q == 0 && ix[q] == 0)) {
                        err = path + ":" + std::to_string(lineNo) + ": index out of range";
                        return false;
                    }
                }
                const std::array<int64_t, 3> key = {ix[0], ix[1], ix[2]};
                auto it = vmap.find(key);
                uint32_t v;
                if (it == vmap.end()) {
                    v = uint32_t(vertPos.size());
                    vmap[key] = v;
                    vertPos.push_back(ix[0] - 1);
                    const float* p = &P[size_t(ix[0] - 1) * 3];
                    m.pos.insert(m.pos.end(), {p[0], p[1], p[2]});
                    if (ix[1] > 0)
                        m.uv.insert(m.uv.end(), {T[size_t(ix[1] - 1) * 2], T[size_t(ix[1] - 1) * 2 + 1]});
                    else
                        m.uv.insert(m.uv.end(), {0.f, 0.f});
                    if (ix[2] > 0) {
                        const float* n = &N[size_t(ix[2] - 1) * 3];
                        m.nrm.insert(m.nrm.end(), {n[0], n[1], n[2]});
                    } else {
                        m.nrm.insert(m.nrm.end(), {0.f, 0.f, 0.f});
                    }
                    hasNormal.push_back(ix[2] > 0);
                } else {
                    v = it->second;
                }
                face.push_back(v);
            }
            for (size_t q = 2; q < face.size(); ++q) {
                m.idx.insert(m.idx.end(), {face[0], face[q - 1], face[q]});
                m.matIdx.push_back(curMat);
            }
        }
    }
    if (!anyMat && m.mats.empty())
        m.mats.push_back(MaterialRec{});
    for (uint32_t& mi : m.matIdx)
        if (mi >= m.mats.size())
            mi = 0;
    std::vector<float> smooth;
    smooth_normals(m.pos, m.idx, vertPos, P.size() / 3, smooth);
    for (size_t v = 0; v < vertPos.size(); ++v)
        if (!hasNormal[v])
            std::copy(&smooth[3 * v], &smooth[3 * v] + 3, &m.nrm[3 * v]);
    return true;
}

// ------------------------------------------------------------------ JSON reads
// The Read helpers of JsonHelpers.cpp: a member of the right type, else nothing.
bool read_number(const json::Value& o, const char* key, float& out)
{
    const json::Value* v = o.find(key);
    if (!v || !v->is_number())
        return false;
    out = float(v->num);
    return true;
}
bool read_int(const json::Value& o, const char* key, int& out)
{
    const json::Value* v = o.find(key);
    if (!v || !v->is_number() || !v->integral || std::fabs(v->num) > 2147483647.0)
        return false;
    out = int(v->num);
    return true;
}
bool read_bool(const json::Value& o, const char* key, bool& out)
{
    const json::Value* v = o.find(key);
    if (!v || !v->is_bool())
        return false;
    out = v->b;
    return true;
}
bool read_string(const json::Value& o, const char* key, std::string& out)
{
    const json::Value* v = o.find(key);
    if (!v || !v->is_string())
        return false;
    out = v->str;
    return true;
}
bool read_floats(const json::Value& o, const char* key, float* out, size_t n)
{
    const json::Value* v = o.find(key);
    if (!v || !v->is_array() || v->items.size() != n)
        return false;
    for (const json::Value& e : v->items)
        if (!e.is_number())
            return false;
    for (size_t k = 0; k < n; ++k)
        out[k] = float(v->items[k].num);
    return true;
}

// float3x4 of LinearMath.h:205-232 (basis vectors x, y, z and translation t)
// with its composition transform(a, b) (:238-262), rotations (:309-351), scale
// and translation (:384-430): the operations instance transforms are built from.
struct M34 {
    float x[3], tx, y[3], ty, z[3], tz;
};
M34 m34_identity() { return M34{{1, 0, 0}, 0, {0, 1, 0}, 0, {0, 0, 1}, 0}; }
float dot3(const float* a, const float* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
M34 m34_mul(const M34& a, const M34& b)
{
    const float t[3] = {a.tx, a.ty, a.tz};
    const float bx[3] = {b.x[0], b.y[0], b.z[0]};
    const float by[3] = {b.x[1], b.y[1], b.z[1]};
    const float bz[3] = {b.x[2], b.y[2], b.z[2]};
    M34 r;
    r.x[0] = dot3(a.x, bx); r.x[1] = dot3(a.x, by); r.x[2] = dot3(a.x, bz);
    r.y[0] = dot3(a.y, bx); r.y[1] = dot3(a.y, by); r.y[2] = dot3(a.y, bz);
    r.z[0] = dot3(a.z, bx); r.z[1] = dot3(a.z, by); r.z[2] = dot3(a.z, bz);
    r.tx = dot3(t, bx) + b.tx;
    r.ty = dot3(t, by) + b.ty;
    r.tz = dot3(t, bz) + b.tz;
    return r;
}
M34 m34_rotate(int axis, float a)
{
    const float s = std::sin(a), c = std::cos(a);
    M34 m = m34_identity();
    if (axis == 0) {
        m.y[1] = c; m.y[2] = s; m.z[1] = -s; m.z[2] = c;
    } else if (axis == 1) {
        m.x[0] = c; m.x[2] = -s; m.z[0] = s; m.z[2] = c;
    } else {
        m.x[0] = c; m.x[1] = s; m.y[0] = -s; m.y[1] = c;
    }
    return m;
}

// helper_math's host normalize (v * 1/sqrt(v.v)) and cross
void normalize3(float* v)
{
    const float r = 1.0f / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= r; v[1] *= r; v[2] *= r;
}
void cross3(const float* a, const float* b, float* out)
{
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

// absolute, lexically normal form of a path (GlobalPath): "." and ".." folded
std::string global_path(const std::string& base, const std::string& p)
{
    const std::string full = join(base, p);
    std::vector<std::string> parts;
    std::string cur;
    for (size_t i = 0; i <= full.size(); ++i) {
        if (i == full.size() || full[i] == '/') {
            if (cur == "..") {
                if (!parts.empty())
                    parts.pop_back();
            } else if (!cur.empty() && cur != ".") {
                parts.push_back(cur);
            }
            cur.clear();
        } else {
            cur += full[i];
        }
    }
    std::string out;
    for (const std::string& q : parts)
        out += "/" + q;
    return out.empty() ? std::string("/") : out;
}

}  // namespace

// ------------------------------------------------------------------ the loaded scene
struct SceneFileObj {
    std::string base;   // where relative paths and cache/ resolve
    std::vector<ModelData> models;   // meshes in first use among the instances
    std::vector<std::string> meshNames, instanceNames, materialNames;
    std::vector<tr_mesh_desc> meshes;
    std::vector<uint32_t> offsets;
    std::vector<tr_instance_desc> instances;
    std::vector<tr_material_desc> materials;
    std::vector<TextureData> textures;
    std::vector<std::string> texturePaths;
    std::vector<tr_texture_desc> texDescs;
    std::vector<uint32_t> materialTextures;
    std::vector<const char*> meshNamePtrs, instanceNamePtrs, materialNamePtrs;
    std::string warnings;
    tr_scene_desc desc{};
    tr_scene_file_info info{};

    // TextureFile::Import (TextureFile.cpp:120-175): one texture per global path;
    // the texture cache format is read from the file itself or from its cache
    // file. Returns the texture's index, or -1 when it cannot be read (the
    // property then has no texture, as when the reference's image import fails).
    int32_t texture(const std::string& path)
    {
        const std::string g = global_path(base, path);
        for (size_t i = 0; i < texturePaths.size(); ++i)
            if (texturePaths[i] == g)
                return int32_t(i);
        std::vector<char> buf;
        TextureData t;
        std::string err;
        bool ok = read_file(g, buf) && read_texture_cache(buf, t, err);
        if (!ok) {
            const std::string c = cache_path(base, g);
            int64_t tc = 0, tf = 0;
            const bool fresh = file_time(c, tc) && (!file_time(g, tf) || tf <= tc);
            ok = fresh && read_file(c, buf) && read_texture_cache(buf, t, err);
        }
        if (!ok) {
            warnings += "texture \"" + g + "\": not a texture cache file and no cache file for it\n";
            return -1;
        }
        textures.push_back(std::move(t));
        texturePaths.push_back(g);
        return int32_t(textures.size() - 1);
    }

    // ModelFile::Import (ModelFile.cpp:331-449): the model cache format from the
    // file itself or its cache file (LoadFromCache's write-time rule), else OBJ.
    bool model(const std::string& path, ModelData& m, std::string& err)
    {
        const std::string g = global_path(base, path);
        std::vector<char> buf;
        if (read_file(g, buf) && header_is(buf, kModelId, kCacheVersion))
            return read_model_cache(buf, m, err);
        const std::string c = cache_path(base, g);
        int64_t tc = 0, tf = 0;
        if (file_time(c, tc) && (!file_time(g, tf) || tf <= tc) && read_file(c, buf) &&
            header_is(buf, kModelId, kCacheVersion))
            return read_model_cache(buf, m, err);
        const size_t dot = g.find_last_of('.');
        if (dot != std::string::npos && lower(g.substr(dot)) == ".obj")
            return read_obj(g, m, err);
        err = "cannot import \"" + g + "\": neither a model cache file nor OBJ";
        return false;
    }
};

}  // namespace tr

using tr::SceneFileObj;

namespace {

tr_status load_scene(const std::string& path, const std::string& base, SceneFileObj& S)
{
    using namespace tr;
    std::vector<char> text;
    if (!read_file(path, text))
        return sf_fail(TR_ERR_INVALID_ARGUMENT, "cannot read \"" + path + "\"");
    json::Value doc;
    std::string err;
    if (!json::parse(std::string(text.begin(), text.end()), doc, err) || !doc.is_object())
        return sf_fail(TR_ERR_INVALID_ARGUMENT,
                       "\"" + path + "\" does not contain valid json" + (err.empty() ? "" : ": " + err));
    S.base = base;

    // ParseModels (SceneFile.cpp:256-284): name -> path, the last declaration wins
    std::map<std::string, std::string> declared;
    if (const json::Value* ms = doc.find("models"); ms && ms->is_array())
        for (const json::Value& m : ms->items) {
            std::string name, mpath;
            if (read_string(m, "name", name) && read_string(m, "path", mpath))
                declared[name] = mpath;
        }

    // ParseInstances (SceneFile.cpp:133-188): model, name, transform operations
    struct Inst {
        std::string name, model;
        M34 xf;
    };
    std::vector<Inst> insts;
    if (const json::Value* is = doc.find("instances"); is && is->is_array())
        for (const json::Value& j : is->items) {
            Inst in;
            if (!read_string(j, "model", in.model))
                continue;
            in.name = in.model;
            read_string(j, "name", in.name);
            in.xf = m34_identity();
            if (const json::Value* ops = j.find("transform"); ops && ops->is_array())
                for (const json::Value& op : ops->items) {
                    float f, f3[3], m12[12];
                    if (read_floats(op, "matrix", m12, 12)) {
                        const M34 m{{m12[0], m12[1], m12[2]}, m12[9], {m12[3], m12[4], m12[5]}, m12[10],
                                    {m12[6], m12[7], m12[8]}, m12[11]};
                        in.xf = m34_mul(in.xf, m);
                    } else if (read_floats(op, "translate", f3, 3)) {
                        M34 m = m34_identity();
                        m.tx = f3[0]; m.ty = f3[1]; m.tz = f3[2];
                        in.xf = m34_mul(in.xf, m);
                    } else if (read_number(op, "rotate-x", f)) {
                        in.xf = m34_mul(in.xf, m34_rotate(0, f * kDegToRad));
                    } else if (read_number(op, "rotate-y", f)) {
                        in.xf = m34_mul(in.xf, m34_rotate(1, f * kDegToRad));
                    } else if (read_number(op, "rotate-z", f)) {
                        in.xf = m34_mul(in.xf, m34_rotate(2, f * kDegToRad));
                    } else if (read_number(op, "scale", f)) {
                        M34 m = m34_identity();
                        m.x[0] = f; m.y[1] = f; m.z[2] = f;
                        in.xf = m34_mul(in.xf, m);
                    } else if (read_floats(op, "scale", f3, 3)) {
                        M34 m = m34_identity();
                        m.x[0] = f3[0]; m.y[1] = f3[1]; m.z[2] = f3[2];
                        in.xf = m34_mul(in.xf, m);
                    }
                }
            insts.push_back(in);
        }

    // ImportModels (SceneFile.cpp:413-441): every declared model an instance names;
    // instances of undeclared or unreadable models are left out
    std::map<std::string, ModelData> imported;
    std::set<std::string> failed;
    for (const Inst& in : insts) {
        auto d = declared.find(in.model);
        if (d == declared.end() || imported.count(in.model))
            continue;
        ModelData m;
        if (!S.model(d->second, m, err)) {
            // ModelFile::Import returns nothing: the model's instances are left out
            S.warnings += "model \"" + in.model + "\": " + err + "\n";
            failed.insert(in.model);
            imported.emplace(in.model, ModelData{});
            continue;
        }
        m.name = in.model;
        imported.emplace(in.model, std::move(m));
    }

    // ParseMaterials (SceneFile.cpp:195-252): per model, per material name, the
    // properties by lower-case MaterialPropertyIds name and "<name>Map" textures
    if (const json::Value* mm = doc.find("materials"); mm && mm->is_array())
        for (const json::Value& jm : mm->items) {
            std::string mname;
            if (!read_string(jm, "model", mname))
                continue;
            auto it = imported.find(mname);
            const json::Value* list = jm.find("materials");
            if (it == imported.end() || failed.count(mname) || !list || !list->is_array())
                continue;
            for (const json::Value& jmat : list->items) {
                std::string matName;
                if (!read_string(jmat, "name", matName))
                    continue;
                MaterialRec* rec = nullptr;
                for (MaterialRec& r : it->second.mats)
                    if (r.name == matName) {
                        rec = &r;
                        break;
                    }
                if (!rec)
                    continue;
                for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                    float f, f3[3];
                    // a number sets the colour's first channel, three numbers the colour
                    if (read_number(jmat, kPropNames[p], f))
                        rec->color[p][0] = f;
                    if (read_floats(jmat, kPropNames[p], f3, 3))
                        std::copy(f3, f3 + 3, rec->color[p]);
                    std::string tex;
                    if (read_string(jmat, (std::string(kPropNames[p]) + "Map").c_str(), tex) && (kPropKinds[p] & kTex))
                        rec->tex[p] = tex;
                }
            }
        }

    // meshes in first use among the instances, materials concatenated per mesh
    // (Renderer::BuildMaterials, Renderer.cpp:378-410)
    std::map<std::string, uint32_t> meshOf;
    uint32_t offset = 0;
    for (const Inst& in : insts) {
        auto it = imported.find(in.model);
        if (it == imported.end() || failed.count(in.model))
            continue;
        if (!meshOf.count(in.model)) {
            meshOf[in.model] = uint32_t(S.models.size());
            S.offsets.push_back(offset);
            offset += uint32_t(it->second.mats.size());
            S.models.push_back(it->second);
            S.meshNames.push_back(in.model);
        }
        tr_instance_desc d{};
        d.mesh = meshOf[in.model];
        // OptixInstance::transform is the float3x4 copied as it lies (Instance.cpp:39-49)
        const float rows[12] = {in.xf.x[0], in.xf.x[1], in.xf.x[2], in.xf.tx, in.xf.y[0], in.xf.y[1],
                                in.xf.y[2], in.xf.ty, in.xf.z[0], in.xf.z[1], in.xf.z[2], in.xf.tz};
        std::copy(rows, rows + 12, d.transform);
        S.instances.push_back(d);
        S.instanceNames.push_back(in.name);
    }
    bool anyTexture = false;
    for (const ModelData& m : S.models)
        for (const MaterialRec& r : m.mats) {
            S.materials.push_back(to_desc(r));
            S.materialNames.push_back(r.name);
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                const int32_t t = r.tex[p].empty() ? -1 : S.texture(r.tex[p]);
                S.materialTextures.push_back(t < 0 ? TR_NO_TEXTURE : uint32_t(t));
                anyTexture |= t >= 0;
            }
        }
    for (const ModelData& m : S.models) {
        tr_mesh_desc d{};
        d.positions = m.pos.data();
        d.normals = m.nrm.data();
        d.texcoords = m.uv.data();
        d.vertex_count = uint32_t(m.pos.size() / 3);
        d.triangle_count = uint32_t(m.idx.size() / 3);
        d.indices = m.idx.data();
        d.material_indices = m.matIdx.data();
        S.meshes.push_back(d);
    }
    for (const TextureData& t : S.textures)
        S.texDescs.push_back(tr_texture_desc{t.w, t.h, t.texels.data()});

    tr_scene_desc& sd = S.desc;
    sd.materials = S.materials.data();
    sd.material_count = uint32_t(S.materials.size());
    sd.instance_count = uint32_t(S.instances.size());
    sd.meshes = S.meshes.data();
    sd.mesh_material_offsets = S.offsets.data();
    sd.instances = S.instances.data();
    sd.mesh_count = uint32_t(S.meshes.size());
    sd.texture_count = anyTexture ? uint32_t(S.texDescs.size()) : 0u;
    sd.textures = anyTexture ? S.texDescs.data() : nullptr;
    sd.material_textures = anyTexture ? S.materialTextures.data() : nullptr;

    tr_scene_file_info& info = S.info;
    info.scene = S.instances.empty() ? nullptr : &S.desc;
    info.mesh_count = sd.mesh_count;
    info.instance_count = sd.instance_count;
    for (const std::string& n : S.meshNames)
        S.meshNamePtrs.push_back(n.c_str());
    for (const std::string& n : S.instanceNames)
        S.instanceNamePtrs.push_back(n.c_str());
    for (const std::string& n : S.materialNames)
        S.materialNamePtrs.push_back(n.c_str());
    info.mesh_names = S.meshNamePtrs.data();
    info.instance_names = S.instanceNamePtrs.data();
    info.material_names = S.materialNamePtrs.data();
    info.warnings = S.warnings.c_str();

    // ParseCamera (SceneFile.cpp:89-128) and CameraNode::Transform (CameraNode.cpp:49-63)
    float pos[3] = {0, 0, -1}, target[3] = {0, 0, 0}, up[3] = {0, 1, 0};
    float aperture = 0, distortion = 0, focalDist = 1e5f, fov = 90.f, bokehRotation = 0;
    int bokehSides = 0;
    if (const json::Value* cam = doc.find("camera")) {
        read_floats(*cam, "position", pos, 3);
        read_floats(*cam, "target", target, 3);
        read_floats(*cam, "up", up, 3);
        read_number(*cam, "aperture", aperture);
        read_number(*cam, "distortion", distortion);
        read_number(*cam, "focaldist", focalDist);
        read_number(*cam, "fov", fov);
        read_number(*cam, "bokehrotation", bokehRotation);
        read_int(*cam, "bokehsides", bokehSides);
    }
    fov = std::fmin(std::fmax(fov, .1f), 179.9f);
    if (pos[0] == target[0] && pos[1] == target[1] && pos[2] == target[2])
        target[2] = pos[2] + 1.f, target[0] = pos[0], target[1] = pos[1];
    normalize3(up);
    float fwd[3] = {target[0] - pos[0], target[1] - pos[1], target[2] - pos[2]}, side[3], up2[3];
    normalize3(fwd);
    cross3(fwd, up, side);
    normalize3(side);
    cross3(side, fwd, up2);
    normalize3(up2);
    tr_camera& c = info.camera;
    std::copy(pos, pos + 3, c.position);
    std::copy(side, side + 3, c.side);
    std::copy(up2, up2 + 3, c.up);
    std::copy(fwd, fwd + 3, c.forward);
    c.aperture = aperture;
    c.distortion = distortion;
    c.focal_dist = focalDist;
    c.fov = fov * kDegToRad;
    c.bokeh_side_count = bokehSides;
    c.bokeh_rotation = bokehRotation;
    std::copy(target, target + 3, info.camera_target);
    std::copy(up, up + 3, info.camera_up);

    // ParseRenderSettings (SceneFile.cpp:351-376) over Renderer::DefaultSettings
    tr_kernel_settings& st = info.settings;
    st = tr_kernel_settings{1u, TR_MAX_DEPTH, 0u, 1e-3f, 1u, 0u, 10.f, 0u};
    info.ao_dist = 1.f;
    info.z_depth_max = 1.f;
    if (const json::Value* r = doc.find("renderer")) {
        int i;
        if (read_int(*r, "multisample", i))
            st.multi_sample = uint32_t(i);
        if (read_int(*r, "maxdepth", i))
            st.max_depth = uint32_t(i);
        read_number(*r, "aodist", info.ao_dist);
        read_number(*r, "zdepthmax", info.z_depth_max);
        read_number(*r, "ray-epsilon", st.ray_epsilon);
    }

    // ParseSkySettings (SceneFile.cpp:380-409) over Sky's defaults (Sky.h:55-67)
    tr_sky_desc& sky = info.sky;
    sky = tr_sky_desc{1u, 1u, {0.f, 1.f, 0.f}, 32.f, 1000.f, 4.f, 1.f};
    if (const json::Value* j = doc.find("sky")) {
        bool b;
        float f, d[3];
        if (read_bool(*j, "enabled", b))
            sky.enabled = b;
        if (read_bool(*j, "drawsun", b))
            sky.draw_sun = b;
        if (read_floats(*j, "dir", d, 3))
            std::copy(d, d + 3, sky.sun_dir);
        if (read_number(*j, "angulardiameter", f))
            sky.sun_angular_diameter = f;
        if (read_number(*j, "intensity", f))
            sky.sun_intensity = f;
        if (read_number(*j, "turbidity", f))
            sky.turbidity = f;
        if (read_number(*j, "bias", f))
            sky.selection_bias = f;
    }
    return TR_OK;
}

}  // namespace

extern "C" {

tr_status tr_scene_file_load(const char* path, const char* base_dir, void** out_file)
{
    if (!path || !out_file)
        return tr::sf_fail(TR_ERR_INVALID_ARGUMENT, "null argument");
    *out_file = nullptr;
    std::unique_ptr<SceneFileObj> S(new (std::nothrow) SceneFileObj());
    if (!S)
        return tr::sf_fail(TR_ERR_OUT_OF_MEMORY, "out of host memory");
    const std::string base = base_dir ? std::string(base_dir) : tr::current_dir();
    try {
        const tr_status st = load_scene(tr::join(base, path), base, *S);
        if (st != TR_OK)
            return st;
    } catch (const std::bad_alloc&) {
        return tr::sf_fail(TR_ERR_OUT_OF_MEMORY, "out of host memory");
    } catch (const std::exception& e) {
        return tr::sf_fail(TR_ERR_INVALID_ARGUMENT, e.what());
    }
    *out_file = S.release();
    return TR_OK;
}

tr_status tr_scene_file_get_info(void* file, tr_scene_file_info* out)
{
    if (!file || !out)
        return tr::sf_fail(TR_ERR_INVALID_ARGUMENT, "null argument");
    *out = static_cast<SceneFileObj*>(file)->info;
    return TR_OK;
}

tr_status tr_scene_file_free(void* file)
{
    delete static_cast<SceneFileObj*>(file);
    return TR_OK;
}

const char* tr_scene_file_last_error(void) { return tr::g_error.c_str(); }

tr_status tr_model_cache_write(const char* path, const tr_mesh_desc* mesh, const tr_material_desc* materials,
                               const char* const* material_names, const char* const* texture_paths,
                               uint32_t material_count)
{
    using namespace tr;
    if (!path || !mesh || (material_count && (!materials || !material_names)))
        return sf_fail(TR_ERR_INVALID_ARGUMENT, "null argument");
    const tr_mesh_desc& m = *mesh;
    if (m.triangle_count && (!m.positions || !m.indices || !m.material_indices))
        return sf_fail(TR_ERR_INVALID_ARGUMENT, "mesh arrays missing");
    ModelData d;
    const size_t nv = m.vertex_count;
    d.pos.assign(m.positions, m.positions + 3 * nv);
    // the reference's cache always holds normals (its importer generates smooth ones) and
    // texcoords (zero where absent)
    if (m.normals) {
        d.nrm.assign(m.normals, m.normals + 3 * nv);
    } else {
        std::vector<int64_t> self(nv);
        for (size_t v = 0; v < nv; ++v)
            self[v] = int64_t(v);
        smooth_normals(d.pos, std::vector<uint32_t>(m.indices, m.indices + 3 * size_t(m.triangle_count)), self, nv,
                       d.nrm);
    }
    d.uv = m.texcoords ? std::vector<float>(m.texcoords, m.texcoords + 2 * nv) : std::vector<float>(2 * nv, 0.f);
    d.idx.assign(m.indices, m.indices + 3 * size_t(m.triangle_count));
    d.matIdx.assign(m.material_indices, m.material_indices + m.triangle_count);
    for (uint32_t i = 0; i < material_count; ++i) {
        MaterialRec r = from_desc(materials[i], material_names[i]);
        if (texture_paths)
            for (uint32_t p = 0; p < TR_PROP_COUNT; ++p) {
                const char* t = texture_paths[size_t(i) * TR_PROP_COUNT + p];
                if (t && (kPropKinds[p] & kTex))
                    r.tex[p] = t;
            }
        d.mats.push_back(std::move(r));
    }
    Writer w;
    write_model_cache(w, d);
    if (!w.save(path))
        return sf_fail(TR_ERR_INVALID_ARGUMENT, std::string("cannot write \"") + path + "\"");
    return TR_OK;
}

tr_status tr_texture_cache_write(const char* path, uint32_t width, uint32_t height, const uint16_t* texels)
{
    using namespace tr;
    if (!path || !texels || width == 0 || height == 0 || width > 0x7fffffffu || height > 0x7fffffffu)
        return sf_fail(TR_ERR_INVALID_ARGUMENT, "bad texture arguments");
    Writer w;
    const char hdr[4] = {kTextureId[0], kTextureId[1], kTextureId[2], char(kCacheVersion)};
    w.raw(hdr, 4);
    const int32_t res[2] = {int32_t(width), int32_t(height)};
    w.raw(res, sizeof(res));
    w.vec(texels, size_t(width) * height, 4);
    if (!w.save(path))
        return sf_fail(TR_ERR_INVALID_ARGUMENT, std::string("cannot write \"") + path + "\"");
    return TR_OK;
}

}  // extern "C"

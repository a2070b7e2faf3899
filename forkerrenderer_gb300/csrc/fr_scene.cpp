// Host-side scene ingest: .scene / .obj / .mtl / .tga into the flat arrays the
// device path uploads, plus the per-frame matrices.
//
// Every parsing rule follows the reference loader so the same files give the
// same numbers: line handling (Ltrim + istringstream, src/scene.cpp:46-57,
// src/model.cpp:158-163), float parsing by istream >> float, the "g" / "usemtl" /
// "f v/t/n" dialect with fan triangulation (model.cpp:143-255), material keys
// (model.cpp:258-408), textures flipped once by the TGA origin bit
// (tgaimage.cpp:100-101) and once for texture v (model.cpp:423), tangent
// generation (model.cpp:430-476), normalisation (model.cpp:107-138) and the
// PBR flag of the last mesh in name order (model.cpp:52-68). Where the
// reference would dereference null or read out of bounds (a face before any
// "g", an unknown material, an index past the arrays) this loader reports an
// error instead.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "forkerrenderer.h"
#include "fr_aonet.h"
#include "fr_hostmath.h"
#include "fr_scene_internal.h"

namespace
{

using fr::V3;

struct LoadError
{
    int code;
    std::string msg;
};

std::string ltrim(const std::string& s)
{
    size_t start = s.find_first_not_of(" \n\r\t\f\v");
    return (start == std::string::npos) ? "" : s.substr(start);
}

// ---- TGA (tgaimage.cpp:43-168, 334-365) -------------------------------------
#pragma pack(push, 1)
struct TgaHeader
{
    uint8_t idlength, colormaptype, datatypecode;
    uint16_t colormaporigin, colormaplength;
    uint8_t colormapdepth;
    uint16_t x_origin, y_origin, width, height;
    uint8_t bitsperpixel, imagedescriptor;
};
#pragma pack(pop)

bool read_file(const std::string& path, std::vector<uint8_t>& buf)
{
    std::ifstream in(path, std::ios::binary | std::ios::ate);
    if (!in.is_open()) return false;
    const std::streamoff n = in.tellg();
    if (n < 0) return false;
    buf.resize((size_t)n);
    in.seekg(0);
    return n == 0 || (bool)in.read(reinterpret_cast<char*>(buf.data()), n);
}

// TGAImage::ReadTgaFile from a file read in one piece (same checks and errors).
bool read_tga(const std::string& path, fr_host_texture& tex, std::string& why)
{
    std::vector<uint8_t> buf;
    if (!read_file(path, buf))
    {
        why = "cannot open " + path;
        return false;
    }
    TgaHeader h;
    if (buf.size() < sizeof h)
    {
        why = "truncated TGA header: " + path;
        return false;
    }
    std::memcpy(&h, buf.data(), sizeof h);
    const uint8_t* src = buf.data() + sizeof h;
    const uint8_t* end = buf.data() + buf.size();
    int w = h.width, ht = h.height, bpp = h.bitsperpixel >> 3;
    if (w <= 0 || ht <= 0 || (bpp != 1 && bpp != 3 && bpp != 4))
    {
        why = "bad TGA size or depth: " + path;
        return false;
    }
    size_t nbytes = (size_t)bpp * w * ht;
    tex.width = w;
    tex.height = ht;
    tex.bpp = bpp;
    tex.data.assign(nbytes, 0);
    if (h.datatypecode == 2 || h.datatypecode == 3)
    {
        if ((size_t)(end - src) < nbytes)
        {
            why = "truncated TGA data: " + path;
            return false;
        }
        std::memcpy(tex.data.data(), src, nbytes);
    }
    else if (h.datatypecode == 10 || h.datatypecode == 11)
    {
        const size_t pixels = (size_t)w * ht;
        size_t cur = 0;
        uint8_t* dst = tex.data.data();
        while (cur < pixels)
        {
            if (src >= end)
            {
                why = "truncated TGA RLE data: " + path;
                return false;
            }
            const int chunk = *src++;
            const bool run = chunk >= 128;
            const size_t count = run ? (size_t)(chunk - 127) : (size_t)(chunk + 1);
            if (cur + count > pixels)
            {
                why = "too many TGA RLE pixels: " + path;
                return false;
            }
            if (run)
            {
                if ((size_t)(end - src) < (size_t)bpp)
                {
                    why = "truncated TGA RLE data: " + path;
                    return false;
                }
                for (size_t i = 0; i < count; ++i) std::memcpy(dst + (cur + i) * bpp, src, (size_t)bpp);
                src += bpp;
            }
            else
            {
                if ((size_t)(end - src) < count * bpp)
                {
                    why = "truncated TGA RLE data: " + path;
                    return false;
                }
                std::memcpy(dst + cur * bpp, src, count * bpp);
                src += count * bpp;
            }
            cur += count;
        }
    }
    else
    {
        why = "unknown TGA format " + std::to_string((int)h.datatypecode) + ": " + path;
        return false;
    }
    auto flip_v = [&]() {
        size_t line = (size_t)w * bpp;
        std::vector<uint8_t> tmp(line);
        for (int j = 0; j < ht / 2; ++j)
        {
            uint8_t* a = tex.data.data() + j * line;
            uint8_t* b = tex.data.data() + (size_t)(ht - 1 - j) * line;
            std::memcpy(tmp.data(), a, line);
            std::memcpy(a, b, line);
            std::memcpy(b, tmp.data(), line);
        }
    };
    if (!(h.imagedescriptor & 0x20)) flip_v();
    if (h.imagedescriptor & 0x10)
    {
        for (int j = 0; j < ht; ++j)
            for (int i = 0; i < w / 2; ++i)
                for (int t = 0; t < bpp; ++t)
                    std::swap(tex.data[((size_t)j * w + i) * bpp + t],
                              tex.data[((size_t)j * w + (w - 1 - i)) * bpp + t]);
    }
    flip_v();  // Model::loadTexture flips for texture v (flipTexCoordY = true)
    return true;
}

// Runs job(i) for i in [0, n) on up to hardware_concurrency threads.
template <typename Job>
void parallel_for(size_t n, Job job)
{
    const size_t workers = std::min<size_t>(n, std::max(1u, std::thread::hardware_concurrency()));
    if (workers <= 1)
    {
        for (size_t i = 0; i < n; ++i) job(i);
        return;
    }
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (size_t w = 0; w < workers; ++w)
        pool.emplace_back([&]() {
            for (size_t i = next++; i < n; i = next++) job(i);
        });
    for (auto& t : pool) t.join();
}

// ---- model -------------------------------------------------------------------
struct LocalMaterial
{
    fr_material_view m;
};

struct LocalMesh
{
    std::vector<int> v, t, n;
    std::string material;
    bool has_material = false;
};

// Which material slot a texture reference fills.
enum TexSlot : int
{
    kSlotKd = 0,
    kSlotKs,
    kSlotKe,
    kSlotBump,
    kSlotAo,
    kSlotPr,
    kSlotPm
};

struct TexRef
{
    std::string material;
    int slot;
    std::string path;
    bool apply;  // false once a repeated newmtl of the material started it again
};

// One model file parsed on its own (on any thread): vertices, meshes, materials
// with their texture references by path, tangents and normalisation.
struct ParsedModel
{
    std::string path;
    bool normalized = false, genTangent = false;
    V3 pos{0.f, 0.f, 0.f};
    float rotY = 0.f, scale = 0.f;
    std::vector<V3> verts, normals, tangents;
    std::vector<float> uvs;
    std::map<std::string, LocalMesh> meshes;
    std::map<std::string, LocalMaterial> mats;
    std::vector<TexRef> texRefs;
    std::vector<std::string> warnings;
    std::exception_ptr error;
};

void parse_materials(ParsedModel& P, const std::string& dir, const std::string& file)
{
    auto& mats = P.mats;
    std::ifstream in(dir + file);
    if (in.fail())
    {
        P.warnings.push_back("cannot open .mtl " + dir + file);
        return;
    }
    std::string line, name;
    bool have = false;
    auto cur = [&]() -> fr_material_view& {
        if (!have) throw LoadError{FR_ERR_PARSE, "material key before newmtl in " + dir + file};
        return mats[name].m;
    };
    while (!in.eof())
    {
        std::getline(in, line);
        line = ltrim(line);
        std::istringstream iss(line.c_str());
        std::string trash;
        auto vec3 = [&](float* dst) {
            iss >> trash;
            float x = 0.f, y = 0.f, z = 0.f;
            iss >> x >> y >> z;
            dst[0] = x, dst[1] = y, dst[2] = z;
        };
        auto map = [&](int slot) {
            std::string f;
            iss >> trash >> f;
            cur();
            P.texRefs.push_back(TexRef{name, slot, dir + f, true});
        };
        if (line.compare(0, 7, "newmtl ") == 0)
        {
            iss >> trash >> name;
            have = true;
            fr_material_view m;
            std::memset(&m, 0, sizeof m);
            m.pbr_albedo[0] = m.pbr_albedo[1] = m.pbr_albedo[2] = 1.f;
            m.map_kd = m.map_ks = m.map_ke = m.map_bump = m.map_ao = m.map_pr = m.map_pm = -1;
            mats[name].m = m;
            // a repeated newmtl starts that material again: its earlier maps still
            // load (texture order) but no longer fill its slots
            for (TexRef& r : P.texRefs)
                if (r.material == name) r.apply = false;
        }
        else if (line.compare(0, 3, "Ka ") == 0) vec3(cur().ka);
        else if (line.compare(0, 3, "Kd ") == 0)
        {
            vec3(cur().kd);
            std::memcpy(cur().pbr_albedo, cur().kd, sizeof(float) * 3);
        }
        else if (line.compare(0, 3, "Ks ") == 0) vec3(cur().ks);
        else if (line.compare(0, 3, "Ke ") == 0) vec3(cur().ke);
        else if (line.compare(0, 3, "Pr ") == 0)
        {
            float f;
            iss >> trash >> f;
            cur().roughness = f;
        }
        else if (line.compare(0, 3, "Pm ") == 0)
        {
            float f;
            iss >> trash >> f;
            cur().metalness = f;
        }
        else if (line.compare(0, 7, "map_Kd ") == 0) map(kSlotKd);
        else if (line.compare(0, 7, "map_Ks ") == 0) map(kSlotKs);
        else if (line.compare(0, 7, "map_Ke ") == 0) map(kSlotKe);
        else if (line.compare(0, 9, "map_Bump ") == 0 || line.compare(0, 5, "norm ") == 0)
            map(kSlotBump);
        else if (line.compare(0, 7, "map_Ao ") == 0) map(kSlotAo);
        else if (line.compare(0, 7, "map_Pr ") == 0) map(kSlotPr);
        else if (line.compare(0, 7, "map_Pm ") == 0) map(kSlotPm);
    }
}

void parse_model(ParsedModel& P)
{
    const std::string& path = P.path;
    const bool normalized = P.normalized, genTangent = P.genTangent;
    auto& verts = P.verts;
    auto& normals = P.normals;
    auto& uvs = P.uvs;
    auto& meshes = P.meshes;
    auto& tangents = P.tangents;
    std::ifstream in(path);
    if (in.fail()) throw LoadError{FR_ERR_IO, "cannot open model " + path};
    std::string dir;
    size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) dir = path.substr(0, slash + 1);

    auto& mats = P.mats;
    std::string line, meshName;
    bool haveMesh = false;
    while (!in.eof())
    {
        std::getline(in, line);
        line = ltrim(line);
        std::istringstream iss(line.c_str());
        char ch;
        std::string trash;
        if (line.compare(0, 7, "mtllib ") == 0)
        {
            std::string f;
            iss >> trash >> f;
            parse_materials(P, dir, f);
        }
        else if (line.compare(0, 2, "v ") == 0)
        {
            iss >> trash;
            V3 v{0.f, 0.f, 0.f};
            iss >> v.x >> v.y >> v.z;
            verts.push_back(v);
        }
        else if (line.compare(0, 3, "vt ") == 0)
        {
            iss >> trash;
            float u = 0.f, w = 0.f;
            iss >> u >> w;
            uvs.push_back(u);
            uvs.push_back(w);
        }
        else if (line.compare(0, 3, "vn ") == 0)
        {
            iss >> trash;
            V3 n{0.f, 0.f, 0.f};
            iss >> n.x >> n.y >> n.z;
            normals.push_back(n);
        }
        else if (line.compare(0, 2, "g ") == 0)
        {
            iss >> ch >> meshName;
            meshes[meshName] = LocalMesh();  // a repeated name restarts that mesh
            haveMesh = true;
        }
        else if (line.compare(0, 7, "usemtl ") == 0)
        {
            std::string m;
            iss >> trash >> m;
            if (!haveMesh) throw LoadError{FR_ERR_PARSE, "usemtl before any g in " + path};
            if (!mats.count(m)) throw LoadError{FR_ERR_PARSE, "unknown material " + m + " in " + path};
            meshes[meshName].material = m;
            meshes[meshName].has_material = true;
        }
        else if (line.compare(0, 2, "f ") == 0)
        {
            if (!haveMesh) throw LoadError{FR_ERR_PARSE, "face before any g in " + path};
            iss >> ch;
            std::vector<int> fv, ft, fn;
            unsigned int a, b, c;
            while (iss >> a >> ch >> b >> ch >> c)
            {
                fv.push_back((int)(a - 1));
                ft.push_back((int)(b - 1));
                fn.push_back((int)(c - 1));
            }
            // no v/t/n corner: the reference's loop bound vertices.size() - 1 wraps around
            // and it reads past the empty list (model.cpp:233); one or two corners add nothing
            if (fv.empty()) throw LoadError{FR_ERR_PARSE, "face without v/t/n corners in " + path};
            LocalMesh& m = meshes[meshName];
            for (int i = 1; i + 1 < (int)fv.size(); ++i)
            {
                int idx[3] = {0, i, i + 1};
                for (int k : idx)
                {
                    m.v.push_back(fv[k]);
                    m.t.push_back(ft[k]);
                    m.n.push_back(fn[k]);
                }
            }
        }
    }
    const int nv = (int)verts.size(), nt = (int)uvs.size() / 2, nn = (int)normals.size();
    for (auto& kv : meshes)
    {
        if (!kv.second.has_material && !kv.second.v.empty())
            throw LoadError{FR_ERR_PARSE, "mesh " + kv.first + " has no material in " + path};
        for (size_t i = 0; i < kv.second.v.size(); ++i)
            if (kv.second.v[i] < 0 || kv.second.v[i] >= nv || kv.second.t[i] < 0 ||
                kv.second.t[i] >= nt || kv.second.n[i] < 0 || kv.second.n[i] >= nn)
                throw LoadError{FR_ERR_PARSE, "face index out of range in " + path};
    }

    // generateTangents (model.cpp:430-476), before normalisation: here only for a
    // normalised model; the others' tangents are generated from the flat scene
    // (on the GPU at upload, fr_scene_host_tangents for host readers).
    if (genTangent && normalized)
    {
        tangents.assign(verts.size(), V3{0.f, 0.f, 0.f});
        for (auto& kv : meshes)
        {
            const LocalMesh& m = kv.second;
            for (size_t f = 0; f < m.v.size() / 3; ++f)
            {
                int i0 = m.v[3 * f], i1 = m.v[3 * f + 1], i2 = m.v[3 * f + 2];
                V3 e1 = fr::sub3(verts[i1], verts[i0]);
                V3 e2 = fr::sub3(verts[i2], verts[i0]);
                const float* t0 = &uvs[2 * m.t[3 * f]];
                const float* t1 = &uvs[2 * m.t[3 * f + 1]];
                const float* t2 = &uvs[2 * m.t[3 * f + 2]];
                float d1s = t1[0] - t0[0], d1t = t1[1] - t0[1];
                float d2s = t2[0] - t0[0], d2t = t2[1] - t0[1];
                float det = d1s * d2t - d2s * d1t;
                if (det == 0.f) continue;
                float inv = 1.f / det;
                V3 raw{d2t * e1.x - d1t * e2.x, d2t * e1.y - d1t * e2.y, d2t * e1.z - d1t * e2.z};
                V3 T = fr::normalize3(fr::scale3(raw, inv));
                tangents[i0] = fr::add3(tangents[i0], T);
                tangents[i1] = fr::add3(tangents[i1], T);
                tangents[i2] = fr::add3(tangents[i2], T);
            }
        }
        for (auto& t : tangents)
        {
            if (fr::length3(t) == 0.f) t = V3{1.f, 0.f, 0.f};
            else t = fr::normalize3(t);
        }
    }

    // normalizePositionVertices (model.cpp:107-138), MinFloat max seeds included.
    if (normalized)
    {
        const float MaxF = 3.40282347e+38f, MinF = 1.17549435e-38f;
        float xmin = MaxF, xmax = MinF, ymin = MaxF, ymax = MinF, zmin = MaxF, zmax = MinF;
        for (const V3& v : verts)
        {
            xmin = std::min(xmin, v.x), xmax = std::max(xmax, v.x);
            ymin = std::min(ymin, v.y), ymax = std::max(ymax, v.y);
            zmin = std::min(zmin, v.z), zmax = std::max(zmax, v.z);
        }
        float sf = 2.f / std::max(xmax - xmin, std::max(ymax - ymin, zmax - zmin));
        fr::M4 m = fr::M4::identity();
        m.m[0][0] = m.m[1][1] = m.m[2][2] = sf;
        m.m[0][3] = -(xmax + xmin) / (xmax - xmin);
        m.m[1][3] = -(ymax + ymin) / (ymax - ymin);
        m.m[2][3] = -(zmax + zmin) / (zmax - zmin);
        for (V3& v : verts)
        {
            float in4[4] = {v.x, v.y, v.z, 1.f}, o[3];
            for (int r = 0; r < 3; ++r)
            {
                float s = 0.f;
                for (int k = 0; k < 4; ++k) s += m.m[r][k] * in4[k];
                o[r] = s;
            }
            v = V3{o[0], o[1], o[2]};
        }
    }
}

class Loader
{
public:
    explicit Loader(fr_scene& s) : S(s) {}

    // A texture's index in first-use order (its file is decoded later).
    int texture(const std::string& path)
    {
        auto it = texCache.find(path);
        if (it != texCache.end()) return it->second;
        const int idx = (int)texPaths.size();
        texPaths.push_back(path);
        texCache[path] = idx;
        return idx;
    }

    // Appends a parsed model to the flat scene, in scene order; its texture
    // references are resolved here, in the order the reference loads them.
    void merge(ParsedModel& P)
    {
        for (const std::string& w : P.warnings) S.warnings.push_back(w);
        for (const TexRef& r : P.texRefs)
        {
            const int idx = texture(r.path);
            if (!r.apply) continue;
            fr_material_view& m = P.mats[r.material].m;
            int32_t* slots[] = {&m.map_kd, &m.map_ks, &m.map_ke, &m.map_bump, &m.map_ao, &m.map_pr, &m.map_pm};
            *slots[r.slot] = idx;
        }
        const auto& verts = P.verts;
        const auto& normals = P.normals;
        const auto& uvs = P.uvs;
        const auto& tangents = P.tangents;
        auto& meshes = P.meshes;
        auto& mats = P.mats;
        const bool genTangent = P.genTangent;
        const V3 pos = P.pos;
        const float rotY = P.rotY, scale = P.scale;
        const int nv = (int)verts.size(), nn = (int)normals.size();
        // Append to the flat scene.
        fr_model_view mv;
        std::memset(&mv, 0, sizeof mv);
        mv.position[0] = pos.x, mv.position[1] = pos.y, mv.position[2] = pos.z;
        mv.rotate_y = rotY;
        mv.scale = scale;
        fr::M4 M = fr::make_model(pos, rotY, scale);
        std::memcpy(mv.model_matrix, M.m, sizeof M.m);
        mv.has_tangents = genTangent ? 1 : 0;
        S.tangent_pending.push_back(genTangent && !P.normalized ? 1 : 0);
        mv.first_vertex = (int64_t)S.positions.size() / 3;
        mv.num_vertices = nv;
        mv.first_normal = (int64_t)S.normals.size() / 3;
        mv.num_normals = nn;
        const int64_t firstUv = (int64_t)S.uvs.size() / 2;
        for (const V3& v : verts) S.positions.insert(S.positions.end(), {v.x, v.y, v.z});
        for (size_t i = 0; i < verts.size(); ++i)
        {
            V3 t = genTangent && P.normalized ? tangents[i] : V3{0.f, 0.f, 0.f};
            S.tangents.insert(S.tangents.end(), {t.x, t.y, t.z});
        }
        S.uvs.insert(S.uvs.end(), uvs.begin(), uvs.end());
        for (const V3& n : normals) S.normals.insert(S.normals.end(), {n.x, n.y, n.z});

        std::map<std::string, int> matIndex;
        for (auto& kv : mats)
        {
            matIndex[kv.first] = (int)S.materials.size();
            S.materials.push_back(kv.second.m);
        }
        const int modelIdx = (int)S.models.size();
        mv.first_mesh = (int32_t)S.meshes.size();
        int lastMat = -1;
        for (auto& kv : meshes)
        {
            const LocalMesh& m = kv.second;
            fr_mesh_view me;
            me.model = modelIdx;
            me.material = m.has_material ? matIndex[m.material] : -1;
            me.first_triangle = (int64_t)S.tri_mesh.size();
            me.num_triangles = (int64_t)m.v.size() / 3;
            const int meshIdx = (int)S.meshes.size();
            for (size_t i = 0; i < m.v.size(); ++i)
            {
                S.tri_v.push_back((int32_t)(mv.first_vertex + m.v[i]));
                S.tri_vt.push_back((int32_t)(firstUv + m.t[i]));
                S.tri_vn.push_back((int32_t)(mv.first_normal + m.n[i]));
            }
            for (int64_t f = 0; f < me.num_triangles; ++f) S.tri_mesh.push_back(meshIdx);
            S.meshes.push_back(me);
            if (m.has_material) lastMat = me.material;  // the last mesh decides the PBR flag
        }
        mv.num_meshes = (int32_t)S.meshes.size() - mv.first_mesh;
        S.models.push_back(mv);
        lastMaterial.push_back(lastMat);
    }

    // Decodes every referenced texture (in parallel), keeps the ones that load in
    // first-use order, and gives the materials their final indices (-1 and a
    // warning for a texture that fails, model.cpp:417-421); then the PBR flags.
    void decode_textures()
    {
        std::vector<fr_host_texture> tex(texPaths.size());
        std::vector<std::string> why(texPaths.size());
        std::vector<char> ok(texPaths.size(), 0);
        parallel_for(texPaths.size(), [&](size_t i) { ok[i] = read_tga(texPaths[i], tex[i], why[i]) ? 1 : 0; });
        std::vector<int> final(texPaths.size(), -1);
        for (size_t i = 0; i < texPaths.size(); ++i)
        {
            if (!ok[i])
            {
                S.warnings.push_back(why[i]);
                continue;
            }
            final[i] = (int)S.textures.size();
            S.textures.push_back(std::move(tex[i]));
        }
        for (fr_material_view& m : S.materials)
            for (int32_t* slot : {&m.map_kd, &m.map_ks, &m.map_ke, &m.map_bump, &m.map_ao, &m.map_pr, &m.map_pm})
                if (*slot >= 0) *slot = final[*slot];
        for (size_t i = 0; i < S.models.size(); ++i)
        {
            const int mi = lastMaterial[i];
            const fr_material_view* mat = mi >= 0 ? &S.materials[mi] : nullptr;
            S.models[i].support_pbr = mat && (mat->map_pm >= 0 || mat->map_pr >= 0) ? 1 : 0;
        }
    }

private:
    fr_scene& S;
    std::map<std::string, int> texCache;
    std::vector<std::string> texPaths;
    std::vector<int> lastMaterial;  // per model: the material of its last mesh, or -1
};

void load_scene_file(fr_scene& S, const std::string& path)
{
    std::ifstream in(path);
    if (in.fail()) throw LoadError{FR_ERR_IO, "cannot open scene " + path};
    std::string dir;
    size_t slash = path.find_last_of('/');
    if (slash != std::string::npos) dir = path.substr(0, slash + 1);

    fr_scene_info& I = S.info;
    std::memset(&I, 0, sizeof I);
    I.width = 1280;
    I.height = 800;
    I.ssaa_kernel = 2;
    I.shadow_on = 1;  // Shadow::s_IsShadowOn default (shadow.cpp:9)
    I.perspective = 1;
    bool haveCamera = false, haveLight = false;
    Loader L(S);
    std::vector<ParsedModel> models;
    std::string line;
    while (!in.eof())
    {
        std::getline(in, line);
        line = ltrim(line);
        std::istringstream iss(line.c_str());
        std::string trash;
        if (line.compare(0, 1, "#") == 0) continue;
        if (line.compare(0, 5, "mode ") == 0)
        {
            std::string m;
            iss >> trash >> m;
            I.deferred = (m == "deferred") ? 1 : 0;
        }
        else if (line.compare(0, 7, "screen ") == 0)
        {
            int w = I.width, h = I.height;
            iss >> trash >> w >> h;
            I.width = w;
            I.height = h;
        }
        else if (line.compare(0, 5, "ssaa ") == 0)
        {
            std::string st;
            int k = I.ssaa_kernel;
            iss >> trash >> st >> k;
            I.ssaa_kernel = k;
            I.ssaa_on = (st == "on") ? 1 : 0;
        }
        else if (line.compare(0, 5, "ssao ") == 0)
        {
            std::string st;
            iss >> trash >> st;
            I.ssao_on = (st == "on") ? 1 : 0;
        }
        else if (line.compare(0, 7, "shadow ") == 0)
        {
            std::string st;
            iss >> trash >> st;
            I.shadow_on = (st == "on") ? 1 : 0;
        }
        else if (line.compare(0, 6, "light ") == 0)
        {
            std::string type;
            iss >> trash >> type;
            float p[3] = {0, 0, 0}, c[3] = {0, 0, 0};
            iss >> p[0] >> p[1] >> p[2] >> c[0] >> c[1] >> c[2];
            if (type == "point")
            {
                std::memcpy(I.light_pos, p, sizeof p);
                std::memcpy(I.light_color, c, sizeof c);
                haveLight = true;
            }
            // "dir" lights are parsed by the reference but never used by Render.
        }
        else if (line.compare(0, 7, "camera ") == 0)
        {
            std::string type;
            iss >> trash >> type;
            if (type == "persp") I.perspective = 1;
            else if (type == "ortho") I.perspective = 0;
            else continue;
            float e[3] = {0, 0, 0}, t[3] = {0, 0, 0};
            iss >> e[0] >> e[1] >> e[2] >> t[0] >> t[1] >> t[2];
            std::memcpy(I.eye, e, sizeof e);
            std::memcpy(I.target, t, sizeof t);
            haveCamera = true;
        }
        else if (line.compare(0, 6, "model ") == 0)
        {
            std::string file, b1, b2;
            iss >> trash >> file >> b1 >> b2;
            V3 pos{0.f, 0.f, 0.f};
            float rot = 0.f, scale = 0.f;
            iss >> pos.x >> pos.y >> pos.z >> rot >> scale;
            std::string full = (!file.empty() && file[0] == '/') ? file : dir + file;
            ParsedModel P;
            P.path = full, P.normalized = b1 == "true", P.genTangent = b2 == "true";
            P.pos = pos, P.rotY = rot, P.scale = scale;
            models.push_back(std::move(P));
        }
    }
    // The model files parse independently; they join the scene in scene order, so
    // draw order, texture order and the first error are the sequential loader's.
    parallel_for(models.size(), [&](size_t i) {
        try
        {
            parse_model(models[i]);
        }
        catch (...)
        {
            models[i].error = std::current_exception();
        }
    });
    for (ParsedModel& P : models)
    {
        if (P.error) std::rethrow_exception(P.error);
        L.merge(P);
    }
    L.decode_textures();
    if (!haveCamera) throw LoadError{FR_ERR_PARSE, "scene has no camera line: " + path};
    if (!haveLight) throw LoadError{FR_ERR_PARSE, "scene has no point light: " + path};
    if (I.width <= 0 || I.height <= 0 || (I.ssaa_on && I.ssaa_kernel <= 0))
        throw LoadError{FR_ERR_PARSE, "bad screen / ssaa size in " + path};

    I.num_models = (int32_t)S.models.size();
    I.num_meshes = (int32_t)S.meshes.size();
    I.num_materials = (int32_t)S.materials.size();
    I.num_textures = (int32_t)S.textures.size();
    I.num_vertices = (int64_t)S.positions.size() / 3;
    I.num_uvs = (int64_t)S.uvs.size() / 2;
    I.num_normals = (int64_t)S.normals.size() / 3;
    I.num_triangles = (int64_t)S.tri_mesh.size();
    if (I.num_triangles >= (int64_t)0x7fffffff)
        throw LoadError{FR_ERR_UNSUPPORTED, "more than 2^31-1 triangles"};
    S.texture_views.resize(S.textures.size());
    for (size_t i = 0; i < S.textures.size(); ++i)
    {
        S.texture_views[i].width = S.textures[i].width;
        S.texture_views[i].height = S.textures[i].height;
        S.texture_views[i].bytes_per_pixel = S.textures[i].bpp;
        S.texture_views[i].data = S.textures[i].data.data();
    }
}

void copy_err(char* err, size_t len, const std::string& m)
{
    if (err && len)
    {
        std::snprintf(err, len, "%s", m.c_str());
    }
}

}  // namespace

void fr_scene_host_tangents(fr_scene* s)
{
    std::lock_guard<std::mutex> lock(s->tangent_mutex);
    if (s->host_tangents_done) return;
    // generateTangents per pending model: its meshes' faces in draw order (mesh
    // key order, then face order), each face's tangent added to its three corners.
    for (size_t m = 0; m < s->models.size(); ++m)
    {
        if (!s->tangent_pending[m]) continue;
        const fr_model_view& mv = s->models[m];
        const int64_t v0 = mv.first_vertex, nv = mv.num_vertices;
        std::vector<V3> acc((size_t)nv, V3{0.f, 0.f, 0.f});
        auto P = [&](int i) { return V3{s->positions[3 * i], s->positions[3 * i + 1], s->positions[3 * i + 2]}; };
        for (int32_t me = mv.first_mesh; me < mv.first_mesh + mv.num_meshes; ++me)
        {
            const fr_mesh_view& mesh = s->meshes[me];
            for (int64_t t = mesh.first_triangle; t < mesh.first_triangle + mesh.num_triangles; ++t)
            {
                const int i0 = s->tri_v[3 * t], i1 = s->tri_v[3 * t + 1], i2 = s->tri_v[3 * t + 2];
                const V3 e1 = fr::sub3(P(i1), P(i0)), e2 = fr::sub3(P(i2), P(i0));
                const float* t0 = &s->uvs[2 * (size_t)s->tri_vt[3 * t]];
                const float* t1 = &s->uvs[2 * (size_t)s->tri_vt[3 * t + 1]];
                const float* t2 = &s->uvs[2 * (size_t)s->tri_vt[3 * t + 2]];
                const float d1s = t1[0] - t0[0], d1t = t1[1] - t0[1];
                const float d2s = t2[0] - t0[0], d2t = t2[1] - t0[1];
                const float det = d1s * d2t - d2s * d1t;
                if (det == 0.f) continue;
                const float inv = 1.f / det;
                const V3 raw{d2t * e1.x - d1t * e2.x, d2t * e1.y - d1t * e2.y, d2t * e1.z - d1t * e2.z};
                const V3 T = fr::normalize3(fr::scale3(raw, inv));
                for (int i : {i0, i1, i2}) acc[i - v0] = fr::add3(acc[i - v0], T);
            }
        }
        for (int64_t i = 0; i < nv; ++i)
        {
            V3 t = acc[(size_t)i];
            t = fr::length3(t) == 0.f ? V3{1.f, 0.f, 0.f} : fr::normalize3(t);
            s->tangents[3 * (v0 + i)] = t.x, s->tangents[3 * (v0 + i) + 1] = t.y, s->tangents[3 * (v0 + i) + 2] = t.z;
        }
    }
    s->host_tangents_done = true;
}

extern "C" {

fr_scene* fr_scene_load(const char* scene_path, char* err, size_t errlen)
{
    if (!scene_path)
    {
        copy_err(err, errlen, "null scene path");
        return nullptr;
    }
    std::unique_ptr<fr_scene> s(new fr_scene());
    try
    {
        load_scene_file(*s, scene_path);
    }
    catch (const LoadError& e)
    {
        copy_err(err, errlen, e.msg);
        return nullptr;
    }
    catch (const std::exception& e)
    {
        copy_err(err, errlen, std::string("scene load failed: ") + e.what());
        return nullptr;
    }
    return s.release();
}

void fr_scene_free(fr_scene* scene) { delete scene; }

int fr_scene_get_info(const fr_scene* scene, fr_scene_info* out)
{
    if (!scene || !out) return FR_ERR_INVALID;
    *out = scene->info;
    return FR_OK;
}

int fr_scene_get_view(const fr_scene* s, fr_scene_view* v)
{
    if (!s || !v) return FR_ERR_INVALID;
    fr_scene_host_tangents(const_cast<fr_scene*>(s));  // host readers see every tangent
    v->info = s->info;
    v->models = s->models.data();
    v->meshes = s->meshes.data();
    v->materials = s->materials.data();
    v->textures = s->texture_views.data();
    v->positions = s->positions.data();
    v->uvs = s->uvs.data();
    v->normals = s->normals.data();
    v->tangents = s->tangents.data();
    v->tri_v = s->tri_v.data();
    v->tri_vt = s->tri_vt.data();
    v->tri_vn = s->tri_vn.data();
    v->tri_mesh = s->tri_mesh.data();
    return FR_OK;
}

fr_scene* fr_scene_from_view(const fr_scene_view* v, char* err, size_t errlen)
{
    if (!v)
    {
        copy_err(err, errlen, "null scene view");
        return nullptr;
    }
    const fr_scene_info& I = v->info;
    auto bad = [&](const std::string& m) -> fr_scene* {
        copy_err(err, errlen, "scene view: " + m);
        return nullptr;
    };
    if (I.num_models < 0 || I.num_meshes < 0 || I.num_materials < 0 || I.num_textures < 0 || I.num_vertices < 0 ||
        I.num_uvs < 0 || I.num_normals < 0 || I.num_triangles < 0 || I.num_triangles > INT32_MAX / 3)
        return bad("negative or too large count");
    if (I.width <= 0 || I.height <= 0 || (I.ssaa_on && I.ssaa_kernel <= 0)) return bad("bad frame size");
    const int64_t T = I.num_triangles;
    if ((I.num_models && !v->models) || (I.num_meshes && !v->meshes) || (I.num_materials && !v->materials) ||
        (I.num_textures && !v->textures) || (I.num_vertices && !v->positions) || (I.num_uvs && !v->uvs) ||
        (I.num_normals && !v->normals) || (T && (!v->tri_v || !v->tri_vt || !v->tri_vn || !v->tri_mesh)))
        return bad("null array");
    std::unique_ptr<fr_scene> s(new fr_scene());
    s->info = I;
    s->models.assign(v->models, v->models + I.num_models);
    s->meshes.assign(v->meshes, v->meshes + I.num_meshes);
    s->materials.assign(v->materials, v->materials + I.num_materials);
    s->positions.assign(v->positions, v->positions + 3 * I.num_vertices);
    s->uvs.assign(v->uvs, v->uvs + 2 * I.num_uvs);
    s->normals.assign(v->normals, v->normals + 3 * I.num_normals);
    s->tri_v.assign(v->tri_v, v->tri_v + 3 * T);
    s->tri_vt.assign(v->tri_vt, v->tri_vt + 3 * T);
    s->tri_vn.assign(v->tri_vn, v->tri_vn + 3 * T);
    s->tri_mesh.assign(v->tri_mesh, v->tri_mesh + T);
    for (int64_t k = 0; k < 3 * T; ++k)
        if (s->tri_v[k] < 0 || s->tri_v[k] >= I.num_vertices || s->tri_vt[k] < 0 || s->tri_vt[k] >= I.num_uvs ||
            s->tri_vn[k] < 0 || s->tri_vn[k] >= I.num_normals)
            return bad("triangle corner index out of range");
    for (int64_t t = 0; t < T; ++t)
        if (s->tri_mesh[t] < 0 || s->tri_mesh[t] >= I.num_meshes) return bad("triangle mesh out of range");
    for (const fr_mesh_view& m : s->meshes)
        if (m.model < 0 || m.model >= I.num_models || m.material < -1 || m.material >= I.num_materials ||
            m.first_triangle < 0 || m.num_triangles < 0 || m.first_triangle + m.num_triangles > T)
            return bad("mesh record out of range");
    for (const fr_model_view& m : s->models)
        if (m.first_mesh < 0 || m.num_meshes < 0 || m.first_mesh + m.num_meshes > I.num_meshes ||
            m.first_vertex < 0 || m.num_vertices < 0 || m.first_vertex + m.num_vertices > I.num_vertices ||
            m.first_normal < 0 || m.num_normals < 0 || m.first_normal + m.num_normals > I.num_normals)
            return bad("model record out of range");
    for (const fr_material_view& m : s->materials)
        for (int32_t slot : {m.map_kd, m.map_ks, m.map_ke, m.map_bump, m.map_ao, m.map_pr, m.map_pm})
            if (slot < -1 || slot >= I.num_textures) return bad("material texture slot out of range");
    s->textures.resize(I.num_textures);
    for (int32_t k = 0; k < I.num_textures; ++k)
    {
        const fr_texture_view& tv = v->textures[k];
        const int bpp = tv.bytes_per_pixel;
        if (tv.width < 0 || tv.height < 0 || (bpp != 1 && bpp != 3 && bpp != 4) ||
            (!tv.data && (int64_t)tv.width * tv.height > 0))
            return bad("texture " + std::to_string(k) + " malformed");
        fr_host_texture& h = s->textures[k];
        h.width = tv.width, h.height = tv.height, h.bpp = bpp;
        h.data.assign(tv.data, tv.data + (size_t)tv.width * tv.height * bpp);
    }
    s->texture_views.resize(I.num_textures);
    for (int32_t k = 0; k < I.num_textures; ++k)
        s->texture_views[k] = fr_texture_view{s->textures[k].width, s->textures[k].height, s->textures[k].bpp,
                                              s->textures[k].data.data()};
    // tangents: the caller's (one per vertex), or generated from the faces for the
    // models that ask for them, as the loader does
    s->tangent_pending.assign(s->models.size(), 0);
    if (v->tangents)
    {
        s->tangents.assign(v->tangents, v->tangents + 3 * I.num_vertices);
        s->host_tangents_done = true;
    }
    else
    {
        s->tangents.assign(3 * (size_t)I.num_vertices, 0.f);
        for (size_t m = 0; m < s->models.size(); ++m) s->tangent_pending[m] = s->models[m].has_tangents ? 1 : 0;
    }
    return s.release();
}

int fr_scene_frame_matrices(const fr_scene* s, int32_t shadow_size, fr_frame_matrices* out)
{
    if (!s) return FR_ERR_INVALID;
    return fr_scene_view_matrices(s, s->info.eye, s->info.target, shadow_size, out);
}

int fr_scene_view_matrices(const fr_scene* s, const float eye[3], const float target[3], int32_t shadow_size,
                           fr_frame_matrices* out)
{
    if (!s || !out || !eye || !target) return FR_ERR_INVALID;
    const fr_scene_info& I = s->info;
    std::memset(out, 0, sizeof *out);
    int W = I.ssaa_on ? I.width * I.ssaa_kernel : I.width;
    int H = I.ssaa_on ? I.height * I.ssaa_kernel : I.height;
    float ratio = (float)I.width / I.height;  // Scene::GetRatio (scene.h:17)
    fr::M4 view = fr::make_look_at(fr::V3{eye[0], eye[1], eye[2]}, fr::V3{target[0], target[1], target[2]});
    fr::M4 proj = I.perspective ? fr::make_perspective(45.f, ratio, 0.01f, 20.f)
                                : fr::make_ortho(-1.f * ratio, 1.f * ratio, -1.f, 1.f, 0.01f, 20.f);
    fr::M4 vp = fr::mul(proj, view);
    fr::M4 lview = fr::make_look_at(fr::V3{I.light_pos[0], I.light_pos[1], I.light_pos[2]},
                                    fr::V3{0.f, 0.f, 0.f});
    const float sv = 3.0f;
    fr::M4 lproj = fr::make_ortho(-sv * ratio, sv * ratio, -sv, sv, 0.1f, 20.f);
    fr::M4 ls = fr::mul(lproj, lview);
    fr::M4 vpm = fr::make_viewport(W, H);
    int SW = shadow_size > 0 ? shadow_size : W, SH = shadow_size > 0 ? shadow_size : H;
    fr::M4 svpm = fr::make_viewport(SW, SH);
    std::memcpy(out->view, view.m, 64);
    std::memcpy(out->projection, proj.m, 64);
    std::memcpy(out->view_projection, vp.m, 64);
    std::memcpy(out->light_space, ls.m, 64);
    std::memcpy(out->viewport, vpm.m, 64);
    std::memcpy(out->shadow_viewport, svpm.m, 64);
    out->width = W;
    out->height = H;
    out->shadow_width = SW;
    out->shadow_height = SH;
    return FR_OK;
}

}  // extern "C"

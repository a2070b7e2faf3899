// Drop-in replacement of the reference renderer's src/render.cpp: the functions
// of namespace Render (src/render.h:20-37) run the frame on the GPU through this
// library's C ABI (include/forkerrenderer.h) and leave the results in the
// reference's own ForkerGL:: buffers (src/forkergl.h:41-55), so the reference's
// unchanged main.cpp (src/main.cpp:18-55) and Output module (src/output.cpp:12-86)
// run on top of it. Build: link this file instead of render.cpp with the
// reference's other sources and libforkerrenderer.so (oracle/Makefile.ref,
// target ref_main_gpu).
//
// The reference's Scene (src/scene.h:13-75) is handed over in memory: its models,
// meshes, materials and textures become an fr_scene_view and fr_scene_from_view
// builds the library's scene from it; nothing is parsed twice. Model, Mesh,
// Texture, TGAImage and Buffer keep the arrays this needs private (model.h:43-53,
// mesh.h:52-60, texture.h:55-60, tgaimage.h:135-139, buffer.h:46-92), so they are
// reached through pointers to members formed in explicit template instantiations,
// where access checking does not apply; the reference's files stay untouched.
//
// Configuration comes from the reference's own compile-time and run-time state:
// the shadow mode and tap counts of shaders/shadow.h, Shadow::GetShadowStatus(),
// ForkerGL::GetRenderMode(), the textures' wrap and filter modes; the SSAO
// constants are the reference's (32 samples, radius 0.075, render.cpp:219-258),
// the library's defaults. Errors are reported on stderr and end the process
// with status 1, as the reference's failed checks do.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <vector>

#include "forkerrenderer.h"
#include "render.h"
#include "render_gpu.h"
#include "shadow.h"

namespace
{

// ---- private members of the reference's classes ---------------------------------
// Each tag declares a friend function whose definition, inside the explicit
// instantiation of Reach<Tag, &Class::member>, returns that pointer to member.
template <typename Tag, auto M>
struct Reach
{
    friend auto member_of(Tag) { return M; }
};

#define FR_REACH(TAG, MEMBER)            \
    struct TAG                           \
    {                                    \
        friend auto member_of(TAG);      \
    };                                   \
    template struct Reach<TAG, &MEMBER>;

FR_REACH(ModelMeshes, Model::m_Meshes)
FR_REACH(ModelVerts, Model::m_Verts)
FR_REACH(ModelTexCoords, Model::m_TexCoords)
FR_REACH(ModelNormals, Model::m_Normals)
FR_REACH(ModelTangents, Model::m_Tangents)
FR_REACH(MeshVertIdx, Mesh::m_FaceVertIndices)
FR_REACH(MeshTexCoordIdx, Mesh::m_FaceTexCoordIndices)
FR_REACH(MeshNormalIdx, Mesh::m_FaceNormalIndices)
FR_REACH(TextureImage, Texture::m_Image)
FR_REACH(TextureWrap, Texture::m_WrapMode)
FR_REACH(TextureFilter, Texture::m_FilterMode)
FR_REACH(ImageData, TGAImage::m_Data)
FR_REACH(Buffer1fData, Buffer1f::m_Data)
FR_REACH(Buffer3fData, Buffer3f::m_Data)

template <typename Tag, typename Obj>
auto& get(Obj& o)
{
    return o.*member_of(Tag{});
}

[[noreturn]] void die(const char* what, const char* detail)
{
    std::fprintf(stderr, "[render_gpu] %s: %s\n", what, detail ? detail : "");
    std::exit(1);
}

// ---- Scene -> fr_scene_view ---------------------------------------------------------
struct SceneArrays
{
    fr_scene_view view{};
    std::vector<fr_model_view> models;
    std::vector<fr_mesh_view> meshes;
    std::vector<fr_material_view> materials;
    std::vector<fr_texture_view> textures;
    std::vector<float> positions, uvs, normals, tangents;
    std::vector<int32_t> triV, triT, triN, triMesh;
    std::map<const Texture*, int32_t> textureIndex;
    int wrap = Texture::NoWrap, filter = Texture::Nearest;
};

int32_t texture_slot(SceneArrays& A, const std::shared_ptr<Texture>& t)
{
    if (!t) return -1;
    auto it = A.textureIndex.find(t.get());
    if (it != A.textureIndex.end()) return it->second;
    Texture& tex = *t;
    TGAImage& img = get<TextureImage>(tex);
    std::vector<std::uint8_t>& bytes = get<ImageData>(img);
    fr_texture_view tv{img.GetWidth(), img.GetHeight(), img.GetBytespp(), bytes.data()};
    const int32_t k = (int32_t)A.textures.size();
    A.textures.push_back(tv);
    A.textureIndex[t.get()] = k;
    if (k == 0) A.wrap = get<TextureWrap>(tex), A.filter = get<TextureFilter>(tex);
    return k;
}

// Material and PBRMaterial of a mesh merged into one record, as the library's
// loader reads an .mtl (model.cpp:258-408 fills both from the same lines).
fr_material_view material_of(SceneArrays& A, const Mesh& mesh)
{
    fr_material_view m;
    std::memset(&m, 0, sizeof m);
    m.pbr_albedo[0] = m.pbr_albedo[1] = m.pbr_albedo[2] = 1.f;
    m.map_kd = m.map_ks = m.map_ke = m.map_bump = m.map_ao = m.map_pr = m.map_pm = -1;
    auto put3 = [](float* dst, const Vector3f& v) { dst[0] = v.x, dst[1] = v.y, dst[2] = v.z; };
    std::shared_ptr<const Material> mat = mesh.GetMaterial();
    std::shared_ptr<const PBRMaterial> pbr = mesh.GetPBRMaterial();
    if (mat)
    {
        put3(m.ka, mat->ka), put3(m.kd, mat->kd), put3(m.ks, mat->ks), put3(m.ke, mat->ke);
        m.map_kd = texture_slot(A, mat->diffuseMap);
        m.map_ks = texture_slot(A, mat->specularMap);
        m.map_ke = texture_slot(A, mat->emissiveMap);
        m.map_bump = texture_slot(A, mat->normalMap);
    }
    if (pbr)
    {
        put3(m.pbr_albedo, pbr->albedo);
        m.roughness = pbr->roughness, m.metalness = pbr->metalness;
        if (m.map_kd < 0) m.map_kd = texture_slot(A, pbr->baseColorMap);
        m.map_ao = texture_slot(A, pbr->ambientOcclusionMap);
        m.map_pr = texture_slot(A, pbr->roughnessMap);
        m.map_pm = texture_slot(A, pbr->metalnessMap);
    }
    return m;
}

void marshal(const Scene& scene, SceneArrays& A)
{
    for (unsigned mi = 0; mi < scene.GetModelCount(); ++mi)
    {
        // Scene keeps a null model when Model::Load failed (scene.cpp:171-192 resolves
        // model paths against the working directory); the reference then crashes
        Model* mp = &const_cast<Model&>(scene.GetModel((int)mi));
        if (!mp) die("scene", "a model failed to load (paths are relative to the working directory)");
        Model& model = *mp;
        fr_model_view mv;
        std::memset(&mv, 0, sizeof mv);
        const Matrix4x4f M = scene.GetModelMatrix((int)mi);
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) mv.model_matrix[4 * r + c] = M[r][c];
        mv.has_tangents = model.HasTangents() ? 1 : 0;
        mv.support_pbr = model.SupportPBR() ? 1 : 0;
        const auto& verts = get<ModelVerts>(model);
        const auto& uvs = get<ModelTexCoords>(model);
        const auto& normals = get<ModelNormals>(model);
        const auto& tangents = get<ModelTangents>(model);
        const int64_t v0 = (int64_t)A.positions.size() / 3, t0 = (int64_t)A.uvs.size() / 2,
                      n0 = (int64_t)A.normals.size() / 3;
        mv.first_vertex = v0, mv.num_vertices = (int64_t)verts.size();
        mv.first_normal = n0, mv.num_normals = (int64_t)normals.size();
        for (const Vector3f& p : verts) A.positions.insert(A.positions.end(), {p.x, p.y, p.z});
        for (const Vector2f& t : uvs) A.uvs.insert(A.uvs.end(), {t.x, t.y});
        for (const Vector3f& n : normals) A.normals.insert(A.normals.end(), {n.x, n.y, n.z});
        for (size_t i = 0; i < verts.size(); ++i)
        {
            if (model.HasTangents() && i < tangents.size())
                A.tangents.insert(A.tangents.end(), {tangents[i].x, tangents[i].y, tangents[i].z});
            else
                A.tangents.insert(A.tangents.end(), {0.f, 0.f, 0.f});
        }
        // meshes in the model's std::map key order: the reference's draw order
        mv.first_mesh = (int32_t)A.meshes.size();
        for (auto& kv : get<ModelMeshes>(model))
        {
            Mesh& mesh = *kv.second;
            fr_mesh_view me;
            me.model = (int32_t)mi;
            me.material = (int32_t)A.materials.size();
            A.materials.push_back(material_of(A, mesh));
            me.first_triangle = (int64_t)A.triMesh.size();
            me.num_triangles = mesh.NumFaces();
            const auto& vi = get<MeshVertIdx>(mesh);
            const auto& ti = get<MeshTexCoordIdx>(mesh);
            const auto& ni = get<MeshNormalIdx>(mesh);
            for (int64_t k = 0; k < 3 * me.num_triangles; ++k)
            {
                A.triV.push_back((int32_t)(v0 + vi[k]));
                A.triT.push_back((int32_t)(t0 + ti[k]));
                A.triN.push_back((int32_t)(n0 + ni[k]));
            }
            for (int64_t f = 0; f < me.num_triangles; ++f) A.triMesh.push_back((int32_t)A.meshes.size());
            A.meshes.push_back(me);
        }
        mv.num_meshes = (int32_t)A.meshes.size() - mv.first_mesh;
        A.models.push_back(mv);
    }
    fr_scene_info& I = A.view.info;
    std::memset(&I, 0, sizeof I);
    I.width = scene.GetWidth(), I.height = scene.GetHeight();
    I.deferred = ForkerGL::GetRenderMode() == ForkerGL::Deferred ? 1 : 0;
    I.ssaa_on = scene.IsSSAAOn() ? 1 : 0;
    I.ssaa_kernel = scene.GetSSAAKernelSize();
    I.ssao_on = scene.IsSSAOOn() ? 1 : 0;
    I.shadow_on = Shadow::GetShadowStatus() ? 1 : 0;
    I.perspective = scene.GetProjectionType() == Camera::Perspective ? 1 : 0;
    const Point3f eye = scene.GetCamera().GetPosition(), at = scene.GetCamera().GetLookAt();
    const Vector3f lp = scene.GetPointLight().position;
    const Color3 lc = scene.GetPointLight().color;
    I.eye[0] = eye.x, I.eye[1] = eye.y, I.eye[2] = eye.z;
    I.target[0] = at.x, I.target[1] = at.y, I.target[2] = at.z;
    I.light_pos[0] = lp.x, I.light_pos[1] = lp.y, I.light_pos[2] = lp.z;
    I.light_color[0] = lc.x, I.light_color[1] = lc.y, I.light_color[2] = lc.z;
    I.num_models = (int32_t)A.models.size(), I.num_meshes = (int32_t)A.meshes.size();
    I.num_materials = (int32_t)A.materials.size(), I.num_textures = (int32_t)A.textures.size();
    I.num_vertices = (int64_t)A.positions.size() / 3, I.num_uvs = (int64_t)A.uvs.size() / 2;
    I.num_normals = (int64_t)A.normals.size() / 3, I.num_triangles = (int64_t)A.triMesh.size();
    fr_scene_view& v = A.view;
    v.models = A.models.data(), v.meshes = A.meshes.data(), v.materials = A.materials.data();
    v.textures = A.textures.data();
    v.positions = A.positions.data(), v.uvs = A.uvs.data(), v.normals = A.normals.data();
    v.tangents = A.tangents.data();
    v.tri_v = A.triV.data(), v.tri_vt = A.triT.data(), v.tri_vn = A.triN.data(), v.tri_mesh = A.triMesh.data();
}

// ---- the library's context for the current scene ---------------------------------------
struct Gpu
{
    const Scene* scene = nullptr;
    fr_scene* frScene = nullptr;
    fr_ctx* ctx = nullptr;
    fr_frame_params params{};
} g;

void check(int rc, const char* what)
{
    if (rc < 0) die(what, g.ctx ? fr_last_error(g.ctx) : "");
}

void bind(const Scene& scene)
{
    if (g.scene == &scene) return;
    SceneArrays A;
    marshal(scene, A);
    char err[512] = {0};
    fr_scene* s = fr_scene_from_view(&A.view, err, sizeof err);
    if (!s) die("fr_scene_from_view", err);
    if (!g.ctx)
    {
        fr_config cfg;
        fr_config_defaults(&cfg);
#if defined(SOFT_SHADOW_PCSS)
        cfg.shadow_mode = FR_SHADOW_PCSS;
#elif defined(SOFT_SHADOW_PCF)
        cfg.shadow_mode = FR_SHADOW_PCF;
#else
        cfg.shadow_mode = FR_SHADOW_HARD;
#endif
        cfg.pcf_samples = PCF_NUM_SAMPLES;
        cfg.blocker_samples = PCSS_BLOCKER_SEARCH_NUM_SAMPLES;
        cfg.texture_wrap = A.wrap;
        cfg.texture_filter = A.filter;
        cfg.keep_float_frame = 1;  // FrameBuffer is a float buffer
        g.ctx = fr_create(&cfg, err, sizeof err);
        if (!g.ctx) die("fr_create", err);
    }
    check(fr_upload_scene(g.ctx, s), "fr_upload_scene");
    if (g.frScene) fr_scene_free(g.frScene);
    g.frScene = s;
    g.scene = &scene;
}

// ---- device buffers -> ForkerGL:: ------------------------------------------------------
void fill(Buffer1f& dst, int w, int h, Buffer::InitType init, fr_buffer_id id)
{
    dst = Buffer1f(w, h, init);
    auto& data = get<Buffer1fData>(dst);
    static_assert(sizeof(data[0]) == sizeof(float), "Buffer1f element is one float");
    check((int)fr_download(g.ctx, id, data.data(), data.size() * sizeof(float)), "fr_download");
}

void fill(Buffer3f& dst, int w, int h, fr_buffer_id id)
{
    dst = Buffer3f(w, h, Buffer::Zero);
    auto& data = get<Buffer3fData>(dst);
    static_assert(sizeof(data[0]) == 3 * sizeof(float), "Buffer3f element is three floats");
    check((int)fr_download(g.ctx, id, data.data(), data.size() * 3 * sizeof(float)), "fr_download");
}

int working_width(const Scene& s) { return s.IsSSAAOn() ? s.GetWidth() * s.GetSSAAKernelSize() : s.GetWidth(); }
int working_height(const Scene& s) { return s.IsSSAAOn() ? s.GetHeight() * s.GetSSAAKernelSize() : s.GetHeight(); }

void read_shadow(const Scene& scene)
{
    if (!Shadow::GetShadowStatus()) return;
    fill(ForkerGL::ShadowBuffer, working_width(scene), working_height(scene), Buffer::Zero, FR_BUF_SHADOW);
}

void read_camera(const Scene& scene, bool deferred)
{
    const int W = working_width(scene), H = working_height(scene);
    fill(ForkerGL::DepthBuffer, W, H, Buffer::MaxPositive, FR_BUF_DEPTH);
    fill(ForkerGL::FrameBuffer, W, H, FR_BUF_FRAME_F32);
    if (!deferred) return;
    fill(ForkerGL::NormalGBuffer, W, H, FR_BUF_GB_NORMAL);
    fill(ForkerGL::WorldPosGBuffer, W, H, FR_BUF_GB_POSITION);
    if (Shadow::GetShadowStatus()) fill(ForkerGL::LightSpaceNDCPosGBuffer, W, H, FR_BUF_GB_LIGHTNDC);
    fill(ForkerGL::AlbedoGBuffer, W, H, FR_BUF_GB_ALBEDO);
    fill(ForkerGL::EmissiveGBuffer, W, H, FR_BUF_GB_EMISSIVE);
    fill(ForkerGL::ParamGBuffer, W, H, FR_BUF_GB_PARAM);
    fill(ForkerGL::ShadingTypeGBuffer, W, H, Buffer::Zero, FR_BUF_GB_TYPE);
    fill(ForkerGL::AmbientOcclusionGBuffer, W, H, Buffer::One, FR_BUF_AO);
}

void read_ssaa(const Scene& scene)
{
    if (!scene.IsSSAAOn()) return;
    const int k = scene.GetSSAAKernelSize();
    const int w = working_width(scene) / k, h = working_height(scene) / k;
    std::vector<std::uint8_t> rgb((size_t)w * h * 3);
    check((int)fr_download(g.ctx, FR_BUF_SSAA_U8, rgb.data(), rgb.size()), "fr_download");
    TGAImage img(w, h, TGAImage::RGB);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
        {
            const std::uint8_t* p = &rgb[((size_t)y * w + x) * 3];
            img.Set(x, y, TGAColor(p[0], p[1], p[2]));
        }
    ForkerGL::AntiAliasedImage = img;
}

}  // namespace

fr_ctx* RenderGpuContext() { return g.ctx; }

namespace Render
{

void Preconfigure(const Scene& scene)
{
    // render.cpp:33-38: the reference's viewport and texture modes, then the scene
    // goes to the GPU once
    ForkerGL::SetViewportMatrix(0, 0, working_width(scene), working_height(scene));
    ForkerGL::TextureWrapMode(Texture::NoWrap);
    ForkerGL::TextureFilterMode(Texture::Nearest);
    bind(scene);
}

void Render(const Scene& scene)
{
    bind(scene);
    check(fr_render_frame(g.ctx, &g.params), "fr_render_frame");
    read_shadow(scene);
    read_camera(scene, ForkerGL::GetRenderMode() == ForkerGL::Deferred);
    read_ssaa(scene);
}

void DoShadowPass(const Scene& scene)
{
    bind(scene);
    check(fr_shadow_pass(g.ctx, &g.params), "fr_shadow_pass");
    read_shadow(scene);
}

void DoForwardPass(const Scene& scene)
{
    bind(scene);
    check(fr_forward_pass(g.ctx, &g.params), "fr_forward_pass");
    read_camera(scene, false);
}

void DoGeometryPass(const Scene& scene)
{
    bind(scene);
    check(fr_geometry_pass(g.ctx, &g.params), "fr_geometry_pass");
}

void DoSSAO(const Scene& scene)
{
    bind(scene);
    check(fr_ssao_pass(g.ctx, &g.params), "fr_ssao_pass");
}

void DoLightingPass(const Scene& scene)
{
    bind(scene);
    check(fr_lighting_pass(g.ctx, &g.params), "fr_lighting_pass");
    read_camera(scene, true);
}

void DoSSAA(const Scene& scene)
{
    bind(scene);
    check(fr_ssaa_pass(g.ctx, &g.params), "fr_ssaa_pass");
    read_ssaa(scene);
}

}  // namespace Render

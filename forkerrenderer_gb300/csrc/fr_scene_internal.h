// Host representation behind the opaque fr_scene handle of forkerrenderer.h.
#pragma once

#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "forkerrenderer.h"

struct fr_host_texture
{
    int width = 0, height = 0, bpp = 0;
    std::vector<uint8_t> data;  // TGAImage byte layout after both vertical flips
};

struct fr_scene
{
    fr_scene_info info{};
    std::vector<fr_model_view> models;
    std::vector<fr_mesh_view> meshes;
    std::vector<fr_material_view> materials;
    std::vector<fr_host_texture> textures;
    std::vector<fr_texture_view> texture_views;
    std::vector<float> positions, uvs, normals, tangents;
    std::vector<int32_t> tri_v, tri_vt, tri_vn, tri_mesh;
    std::vector<std::string> warnings;
    // Per model: 1 = its tangents are generated from its faces when first needed
    // (fr_upload_scene on the GPU; fr_scene_get_view on the host), 0 = in `tangents`
    // already (no tangents, or a normalised model: generateTangents runs on the
    // positions before normalisation, which only the loader sees).
    std::vector<uint8_t> tangent_pending;
    bool host_tangents_done = false;
    std::mutex tangent_mutex;
};

// Fills `tangents` of the pending models on the host (generateTangents,
// model.cpp:430-476, from the flat arrays); idempotent and thread-safe.
void fr_scene_host_tangents(fr_scene* s);

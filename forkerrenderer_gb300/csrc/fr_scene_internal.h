// Host representation behind the opaque fr_scene handle of forkerrenderer.h.
#pragma once

#include <cstdint>
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
};

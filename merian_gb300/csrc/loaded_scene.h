// The host arrays of a scene loaded from a file (pbrt_loader.cpp, gltf_loader.cpp), which
// gbpt_loaded_scene_info exposes as a gbpt_scene_desc. Host-only C++.
#pragma once

#include "gbpt.h"

#include <cstdint>
#include <string>
#include <vector>

struct gbpt_loaded_scene {
    std::vector<gbpt_packed_vertex> vertices;
    std::vector<uint32_t> indices;
    std::vector<gbpt_geometry> geometries;
    std::vector<gbpt_material> materials;
    std::vector<gbpt_blas_range> blas;
    std::vector<gbpt_instance> instances;
    std::vector<float> env_texels;
    gbpt_env_map env{};
    bool has_env = false;
    // RGBA8 textures (texels per texture; descriptors point into them)
    std::vector<std::vector<uint8_t>> texels;
    std::vector<gbpt_texture> textures;
    gbpt_camera camera{};
    uint32_t width = 1280, height = 720;
    std::vector<std::string> warnings;
};

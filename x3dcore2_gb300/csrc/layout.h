// Plain-old-data layouts shared by the host packer (C++) and the CUDA kernels.
#pragma once

#include <cstdint>

namespace e8g {

struct DevMaterial {
    uint32_t type; // E8G_MAT_*
    float albedo[3];
    float a, b;   // oren_nayar A, B (material.cpp:113-115)
    float alpha2; // cook_torr 2 r^2 (material.cpp:176)
    float ior_re, ior_im;
    int32_t mix0, mix1;
    float ratio;
    float rough; // the roughness parameter r itself (gradients are taken with respect to it)
    uint32_t pad[3];
};
static_assert(sizeof(DevMaterial) == 64, "DevMaterial is one 64-byte line");

struct DevCamera {
    float origin[3];
    float rot[9];
    float sensor, focal, aspect;
};

} // namespace e8g

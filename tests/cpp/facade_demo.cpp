// Drives the C++ facade the way a Task-layer call site would.
//   facade_demo check   -> argument checks only (no GPU needed)
//   facade_demo render  -> prepare + render a 2-camera fisheye rig on the GPU
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "panostitch.hpp"

static ps_photo_param fisheye(double yaw)
{
    ps_photo_param p;
    std::memset(&p, 0, sizeof p);
    p.image_type = 1;
    p.hfov = 200.0;
    p.yaw = yaw;
    return p;
}

int main(int argc, char** argv)
{
    const bool render = argc > 1 && std::strcmp(argv[1], "render") == 0;
    panostitch::CudaPanoramaRender2 r;
    std::vector<ps_photo_param> cams = {fisheye(0), fisheye(180)};
    // reference preconditions: dst must be even with width == 2 * height
    if (r.prepare(cams, 1, 5, {160, 120}, {250, 128})) return 1;
    if (r.lastError().find("not qualified") == std::string::npos) return 2;
    if (r.getNumImages() != 0) return 3;
    std::vector<unsigned char> frame(160 * 120 * 4, 0);
    std::vector<unsigned char> out(256 * 128 * 4, 1);
    std::vector<ps_image> src = {{frame.data(), 160 * 4, 160, 120, PS_FMT_BGR32, PS_MEM_HOST},
                                 {frame.data(), 160 * 4, 160, 120, PS_FMT_BGR32, PS_MEM_HOST}};
    ps_image dst = {out.data(), 256 * 4, 256, 128, PS_FMT_BGR32, PS_MEM_HOST};
    if (r.render(src, dst)) return 4;  // not prepared
    // decoder frames: NV12 gray (Y 126, U = V = 128 convert to BGR 128)
    std::vector<unsigned char> yp(160 * 120, 126), uvp(160 * 60, 128);
    const ps_planar_image nv12 = {{yp.data(), uvp.data(), nullptr}, {160, 160, 0}, 160, 120, PS_FMT_NV12, PS_MEM_HOST};
    std::vector<ps_planar_image> psrc(2, nv12);
    if (r.renderPlanar(psrc, &dst, nullptr)) return 10;  // not prepared
    // the dual-fisheye render: one frame, two cameras (not prepared yet)
    panostitch::CudaRicohPanoramaRender ricoh;
    if (ricoh.render({src[0]}, dst)) return 14;
    if (ricoh.lastError().find("prepare") == std::string::npos) return 15;
    if (ricoh.getNumImages() != 0) return 16;
    if (!render) {
        std::printf("facade check ok\n");
        return 0;
    }
    if (!r.prepare(cams, 1, 5, {160, 120}, {256, 128})) {
        std::fprintf(stderr, "%s\n", r.lastError().c_str());
        return 5;
    }
    for (size_t i = 0; i < frame.size(); i += 4) frame[i] = frame[i + 1] = frame[i + 2] = 77;
    // malformed LUTs: skipped with a warning, like the reference
    std::vector<std::vector<std::vector<unsigned char>>> bad(2, std::vector<std::vector<unsigned char>>(3));
    if (!r.render(src, dst, bad)) {
        std::fprintf(stderr, "%s\n", r.lastError().c_str());
        return 6;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return 7;
    // a constant frame stitches to the same constant away from the coverage
    // borders (the Laplacian of the masked pyramid is non-zero only there)
    long covered = 0, exact = 0;
    for (size_t i = 0; i < out.size(); i += 4) {
        if (out[i] == 0 && out[i + 1] == 0 && out[i + 2] == 0) continue;
        covered++;
        exact += out[i] == 77 && out[i + 1] == 77 && out[i + 2] == 77;
    }
    if (covered == 0) return 8;
    if (exact < covered * 9 / 10) return 9;
    if (!r.renderPlanar(psrc, &dst, nullptr)) {
        std::fprintf(stderr, "%s\n", r.lastError().c_str());
        return 11;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return 12;
    long covered2 = 0, exact2 = 0;
    for (size_t i = 0; i < out.size(); i += 4) {
        if (out[i] == 0 && out[i + 1] == 0 && out[i + 2] == 0) continue;
        covered2++;
        exact2 += out[i] == 128 && out[i + 1] == 128 && out[i + 2] == 128;
    }
    if (covered2 != covered || exact2 < covered2 * 9 / 10) return 13;
    std::printf("facade render ok: %ld covered pixels, %ld exactly 77; from NV12 %ld exactly 128\n", covered, exact,
                exact2);
    return 0;
}

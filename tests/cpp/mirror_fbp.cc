// Drop-in check of the C++ operator mirror (include/ct_recon/*.h): the fan FBP
// chain written against the reference's class API -- FanWeighting, RampFilterPrep
// + RampFilter, FanBackprojection2DPixDrivenPrep + FanBackprojection2DPixDriven
// and its Grad -- on raw float32 files, as a reference C++ user would call it.
//
//   mirror_fbp <dir> ns na ds orbit offset_s orbit_start nx ny dx dy offset_x offset_y dso dsd
//
// Reads <dir>/sino.f32 ([na][ns]) and <dir>/img_in.f32 ([ny][nx]); writes
// <dir>/recon.f32 ([ny][nx]) and <dir>/grad.f32 ([na][ns]).  Exit code 0 on success.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "ct_recon/bp_fan_2d.h"
#include "ct_recon/fan_weighting.h"
#include "ct_recon/filter.h"

static bool read_file(const char* path, std::vector<float>& v)
{
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    const size_t n = std::fread(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
    return n == v.size();
}

static bool write_file(const char* path, const std::vector<float>& v)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) return false;
    const size_t n = std::fwrite(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
    return n == v.size();
}

int main(int argc, char** argv)
{
    if (argc != 16) {
        std::fprintf(stderr, "usage: mirror_fbp dir ns na ds orbit offset_s orbit_start nx ny dx dy offset_x offset_y dso dsd\n");
        return 2;
    }
    const char* dir = argv[1];
    const unsigned ns = std::atoi(argv[2]), na = std::atoi(argv[3]);
    const double ds = std::atof(argv[4]), orbit = std::atof(argv[5]), offset_s = std::atof(argv[6]);
    const double orbit_start = std::atof(argv[7]);
    const unsigned nx = std::atoi(argv[8]), ny = std::atoi(argv[9]);
    const double dx = std::atof(argv[10]), dy = std::atof(argv[11]);
    const double ox = std::atof(argv[12]), oy = std::atof(argv[13]);
    const double dso = std::atof(argv[14]), dsd = std::atof(argv[15]);

    std::vector<float> sino(static_cast<size_t>(na) * ns), img_in(static_cast<size_t>(nx) * ny);
    char path[4096];
    std::snprintf(path, sizeof(path), "%s/sino.f32", dir);
    if (!read_file(path, sino)) return 3;
    std::snprintf(path, sizeof(path), "%s/img_in.f32", dir);
    if (!read_file(path, img_in)) return 3;

    float *d_sino, *d_w, *d_f, *d_img, *d_in, *d_grad;
    double *d_filter, *d_xpos, *d_ypos, *d_sc;
    const size_t sb = sino.size() * sizeof(float), ib = img_in.size() * sizeof(float);
    if (cudaMalloc(&d_sino, sb) || cudaMalloc(&d_w, sb) || cudaMalloc(&d_f, sb) ||
        cudaMalloc(&d_grad, sb) || cudaMalloc(&d_img, ib) || cudaMalloc(&d_in, ib) ||
        cudaMalloc(&d_filter, (2 * ns + 1) * sizeof(double)) ||
        cudaMalloc(&d_xpos, nx * sizeof(double)) || cudaMalloc(&d_ypos, ny * sizeof(double)) ||
        cudaMalloc(&d_sc, 2 * na * sizeof(double)))
        return 4;
    cudaMemcpy(d_sino, sino.data(), sb, cudaMemcpyHostToDevice);
    cudaMemcpy(d_in, img_in.data(), ib, cudaMemcpyHostToDevice);
    cudaStream_t stream;
    cudaStreamCreate(&stream);

    using namespace ct_recon;
    FanWeighting<float> weighting(FanWeightingParam(ns, na, ds, offset_s, dso, dsd, 1));
    FilterParam fparam(ns, na, ds, dsd, 1);
    RampFilterPrep filter_prep(fparam);
    RampFilter<float> filter(fparam);
    FanBackprojection2DParam bparam(ns, na, ds, orbit, offset_s, orbit_start, nx, ny, dx, dy, ox,
                                    oy, dso, dsd, -1);
    FanBackprojection2DPixDrivenPrep bp_prep(bparam);
    FanBackprojection2DPixDriven<float> bp(bparam);
    FanBackprojection2DPixDrivenGrad<float> bp_grad(bparam);
    const FanBackprojection2D<float>& bp_base = bp;  // reference-style polymorphic use

    bool ok = weighting.calculate_on_gpu(d_sino, d_w, stream) &&
              filter_prep.calculate_on_gpu(d_filter, stream) &&
              filter.calculate_on_gpu(d_w, d_filter, d_f, stream) &&
              bp_prep.calculate_on_gpu(d_xpos, d_ypos, d_sc, stream) &&
              bp_base.calculate_on_gpu(d_f, d_img, d_xpos, d_ypos, d_sc, stream) &&
              bp_grad.calculate_on_gpu(d_in, d_grad, d_xpos, d_ypos, d_sc, stream);
    // the CPU methods are declared for source compatibility and refuse
    ok = ok && !bp.calculate_on_cpu(nullptr, nullptr, nullptr, nullptr, nullptr);
    if (!ok) {
        std::fprintf(stderr, "operator failed: %s\n", ctr_last_error());
        return 5;
    }
    std::vector<float> recon(img_in.size()), grad(sino.size());
    cudaMemcpy(recon.data(), d_img, ib, cudaMemcpyDeviceToHost);
    cudaMemcpy(grad.data(), d_grad, sb, cudaMemcpyDeviceToHost);
    std::snprintf(path, sizeof(path), "%s/recon.f32", dir);
    if (!write_file(path, recon)) return 6;
    std::snprintf(path, sizeof(path), "%s/grad.f32", dir);
    if (!write_file(path, grad)) return 6;
    std::printf("mirror_fbp ok\n");
    return 0;
}

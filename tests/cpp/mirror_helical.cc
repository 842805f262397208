// Drop-in check of the helical mirror (include/ct_recon/helical_interpolation.h):
// HelicalInterpolation360<double> / HelicalInterpolation180<double> called as a
// reference C++ user calls the reference's classes, on a raw float64 file.
//
//   mirror_helical <dir> <360|180> ns nt na ds dt offset_s offset_t orbit_start orbit
//                  couch_begin couch_mov view_per_rot nz dz z0 thickness dso dsd
//
// Reads <dir>/in.f64 ([na][nt][ns]); writes <dir>/out<method>.f64 ([nz][view_per_rot][ns]).
// Prints "runtime_error: <message>" and exits 2 where the class throws.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <vector>

#include <cuda_runtime.h>

#include "ct_recon/helical_interpolation.h"

int main(int argc, char** argv)
{
    if (argc != 21) {
        std::fprintf(stderr, "usage: mirror_helical <dir> <360|180> <18 parameters>\n");
        return 1;
    }
    auto u = [&](int i) { return static_cast<unsigned>(std::strtoul(argv[i], nullptr, 10)); };
    auto d = [&](int i) { return std::strtod(argv[i], nullptr); };
    const ct_recon::HelicalInterpolationParam p(u(3), u(4), u(5), d(6), d(7), d(8), d(9), d(10), d(11), d(12),
                                                d(13), u(14), u(15), d(16), d(17), d(18), d(19), d(20));
    const bool m360 = std::strcmp(argv[2], "360") == 0;
    const size_t n_in = static_cast<size_t>(p.na) * p.nt * p.ns, n_out = static_cast<size_t>(p.nz) * p.view_per_rot * p.ns;
    std::vector<double> in(n_in), out(n_out, 0.0);
    std::string path = std::string(argv[1]) + "/in.f64";
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(in.data(), sizeof(double), n_in, f) != n_in) return 1;
    std::fclose(f);
    double *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, n_in * sizeof(double)) != cudaSuccess || cudaMalloc(&dout, n_out * sizeof(double)) != cudaSuccess)
        return 1;
    cudaMemcpy(din, in.data(), n_in * sizeof(double), cudaMemcpyHostToDevice);
    try {
        const bool ok = m360 ? ct_recon::HelicalInterpolation360<double>(p).calculate_on_gpu(din, dout, nullptr)
                             : ct_recon::HelicalInterpolation180<double>(p).calculate_on_gpu(din, dout, nullptr);
        if (!ok) return 1;
    } catch (const std::runtime_error& e) {
        std::printf("runtime_error: %s\n", e.what());
        return 2;
    }
    cudaMemcpy(out.data(), dout, n_out * sizeof(double), cudaMemcpyDeviceToHost);
    path = std::string(argv[1]) + "/out" + argv[2] + ".f64";
    f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(out.data(), sizeof(double), n_out, f) != n_out) return 1;
    std::fclose(f);
    cudaFree(din);
    cudaFree(dout);
    return 0;
}

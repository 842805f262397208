// Helical rebinning: 3-D helical sinograms to 2-D fan-beam sinograms, one per
// reconstructed slice, by 360LI or 180LI z interpolation (reference
// src/helical_interpolation.cc:80-370, include/helical_interpolation.h).
//
// The reference runs this on the CPU only.  Here one thread computes one
// output sample (slice, view, channel) with the reference's arithmetic: every
// operation is an FP64 intrinsic in the reference's order (__dadd_rn and
// friends, so nothing is contracted into an FMA), row sums accumulate in FP64
// for both T, and the per-channel cos(gamma) and per-slice view ranges come
// from the host (ctr_helical_interpolation_prep) with the reference's own libm
// calls.  The output therefore equals the reference's bit for bit.
//
// Layout: input [na][nt][ns] (view, detector row, channel), output
// [nz][view_per_rot][ns]; a block covers 128 consecutive channels of one
// (slice, view) row, so every row read is a coalesced channel run.
#include <cmath>
#include <vector>

#include "ctr_common.cuh"

namespace ctr {
namespace {

constexpr int kHeliThreads = 128;
constexpr double kHeliPi = 3.14159265358979323846;  // M_PI of the reference's <cmath>

// Device table written by ctr_helical_interpolation_prep: a header, then one
// HeliChan per channel, then one HeliSlice per slice.
struct HeliHeader {
    int method;  // CTR_HELICAL_360 or CTR_HELICAL_180
    unsigned ns, nz, vpr;
};
struct HeliChan {
    double cg;    // cos(gamma), gamma = (is - center_s) * ds / dsd
    double dif;   // 180LI: views back to the complementary ray, (pi - 2 gamma) / orbit
    double sc;    // 180LI: the complementary ray's channel, center_s - s / ds
    double pad;
};
struct HeliSlice {
    double z;                   // slice position, z0 + dz added iz times
    int center, lo, hi, first;  // nearest view, view range [lo, hi], first output view
    int valid;                  // 0: [lo, hi] leaves the scan ("View not enough for this slice!")
    int pad;
};
static_assert(sizeof(HeliHeader) == 16 && sizeof(HeliChan) == 32 && sizeof(HeliSlice) == 32,
              "table layout");

struct HeliGeo {
    unsigned ns, nt, na, vpr, nz;
    double center_t, couch_begin, couch_mov, half_th, dso, dsd, nt_d, ns_last;
    size_t in_item, out_item;
};

// Rows [r0, r1) the thick slice covers for a source z_dif below the slice:
// the slab edges projected onto the detector, clamped to it
// (src/helical_interpolation.cc:105-111).  false when the slab misses.
__device__ __forceinline__ bool heli_rows(const HeliGeo& g, double zd, double cg, int& r0, int& r1)
{
    const double top = __dsub_rn(g.center_t,
                                 __dmul_rn(__dmul_rn(__ddiv_rn(__dadd_rn(zd, g.half_th), g.dso), cg), g.dsd));
    const double bot = __dsub_rn(g.center_t,
                                 __dmul_rn(__dmul_rn(__ddiv_rn(__dsub_rn(zd, g.half_th), g.dso), cg), g.dsd));
    if (bot < 0.0 || top >= g.nt_d) return false;
    r0 = static_cast<int>(floor(top < 0.0 ? 0.0 : top));
    r1 = static_cast<int>(ceil(bot >= g.nt_d ? g.nt_d : bot));
    return true;
}

// Rows in [r0, r1): the reference's loop count (0 for an inverted slab, so
// that its mean is 0/0 as there).
__device__ __forceinline__ double heli_count(int r0, int r1) { return static_cast<double>(r1 > r0 ? r1 - r0 : 0); }

// Mean over rows [r0, r1) of one channel column (stride ns between rows).
template <typename T>
__device__ __forceinline__ double heli_mean(const T* __restrict__ col, unsigned ns, int r0, int r1)
{
    double acc = 0.0;
    for (int r = r0; r < r1; ++r)
        acc = __dadd_rn(acc, static_cast<double>(__ldg(col + static_cast<size_t>(r) * ns)));
    return __ddiv_rn(acc, heli_count(r0, r1));
}

// One sample of a 180LI complementary ray; views outside [0, na) read as 0
// and raise CTR_HELICAL_OUTSIDE (the reference indexes out of bounds there).
template <typename T>
__device__ __forceinline__ double heli_at(const T* __restrict__ in, const HeliGeo& g, int view, int r, int c,
                                          bool& outside)
{
    if (view < 0 || static_cast<unsigned>(view) >= g.na) {
        outside = true;
        return 0.0;
    }
    return static_cast<double>(__ldg(in + (static_cast<size_t>(view) * g.nt + r) * g.ns + c));
}

template <typename T, int M>
__global__ void __launch_bounds__(kHeliThreads)
    helical_kernel(const T* __restrict__ in, T* __restrict__ out, const HeliHeader* __restrict__ tab, HeliGeo g,
                   unsigned* status)
{
    if (tab->method != M || tab->ns != g.ns || tab->nz != g.nz || tab->vpr != g.vpr) {
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
            atomicOr(status, CTR_HELICAL_BAD_TABLE);
        return;
    }
    const unsigned is = blockIdx.x * kHeliThreads + threadIdx.x;
    if (is >= g.ns) return;
    const unsigned iv = blockIdx.y;
    const unsigned iz = blockIdx.z % g.nz, b = blockIdx.z / g.nz;
    const HeliSlice s = reinterpret_cast<const HeliSlice*>(reinterpret_cast<const HeliChan*>(tab + 1) + g.ns)[iz];
    status += blockIdx.z;  // one status word per (item, slice)
    if (!s.valid) {        // the reference throws before touching this slice
        if (is == 0 && iv == 0) atomicOr(status, CTR_HELICAL_NO_VIEWS);
        return;
    }
    const HeliChan c = reinterpret_cast<const HeliChan*>(tab + 1)[is];
    in += b * g.in_item;
    T* o = out + b * g.out_item + (static_cast<size_t>(iz) * g.vpr + iv) * g.ns + is;
    const size_t view_stride = static_cast<size_t>(g.nt) * g.ns;

    const double zrel = __dsub_rn(s.z, g.couch_begin);  // z - couch_begin, then - view * couch_mov
    int cur = s.first + static_cast<int>(iv);
    if (M == CTR_HELICAL_180 && cur > s.hi) cur -= static_cast<int>(g.vpr);
    const double zd = __dsub_rn(zrel, __dmul_rn(static_cast<double>(cur), g.couch_mov));

    int r0 = 0, r1 = 0;
    double vcur = 0.0, vcor = 0.0, zd2;
    const bool ucur = heli_rows(g, zd, c.cg, r0, r1);
    if (ucur) vcur = heli_mean(in + cur * view_stride + is, g.ns, r0, r1);

    bool ucor;
    if (M == CTR_HELICAL_360) {
        // the view one rotation away, on the other side of the slice
        const int cor = cur >= s.center ? cur - static_cast<int>(g.vpr) : cur + static_cast<int>(g.vpr);
        zd2 = __dsub_rn(zrel, __dmul_rn(static_cast<double>(cor), g.couch_mov));
        ucor = heli_rows(g, zd2, c.cg, r0, r1);
        if (ucor) vcor = heli_mean(in + cor * view_stride + is, g.ns, r0, r1);
    } else {
        // the complementary ray: (pi - 2 gamma) / orbit views back, wrapped into [lo, hi] once each way
        double cv = __dsub_rn(static_cast<double>(cur), c.dif);
        if (cv < static_cast<double>(s.lo)) cv = __dadd_rn(cv, static_cast<double>(g.vpr));
        if (cv > static_cast<double>(s.hi)) cv = __dsub_rn(cv, static_cast<double>(g.vpr));
        zd2 = __dsub_rn(zrel, __dmul_rn(cv, g.couch_mov));
        ucor = heli_rows(g, zd2, c.cg, r0, r1);
        if (ucor) {
            const int vl = static_cast<int>(floor(cv)), vr = static_cast<int>(ceil(cv));
            const double u = __dsub_rn(cv, static_cast<double>(vl));
            if (c.sc < 0.0 || c.sc > g.ns_last) {
                *o = static_cast<T>(vcur);  // mirrored channel off the detector: no interpolation
                return;
            }
            const int cl = static_cast<int>(floor(c.sc)), cr = static_cast<int>(ceil(c.sc));
            const double v = __dsub_rn(c.sc, static_cast<double>(cl)), w = __dsub_rn(1.0, v);
            double left = 0.0, right = 0.0;
            bool outside = false;
            for (int r = r0; r < r1; ++r) {
                left = __dadd_rn(left, __dadd_rn(__dmul_rn(w, heli_at(in, g, vl, r, cl, outside)),
                                                 __dmul_rn(v, heli_at(in, g, vl, r, cr, outside))));
                right = __dadd_rn(right, __dadd_rn(__dmul_rn(w, heli_at(in, g, vr, r, cl, outside)),
                                                   __dmul_rn(v, heli_at(in, g, vr, r, cr, outside))));
            }
            if (outside) atomicOr(status, CTR_HELICAL_OUTSIDE);
            vcor = __ddiv_rn(__dadd_rn(__dmul_rn(__dsub_rn(1.0, u), left), __dmul_rn(u, right)),
                             heli_count(r0, r1));
        }
    }

    double val;
    if (ucur && ucor)
        val = __ddiv_rn(__dsub_rn(__dmul_rn(zd, vcor), __dmul_rn(zd2, vcur)), __dsub_rn(zd, zd2));
    else if (ucur)
        val = vcur;
    else if (ucor)
        val = vcor;
    else {
        atomicOr(status, CTR_HELICAL_NO_ROWS);  // the reference throws "No row data available!"
        val = 0.0;
    }
    *o = static_cast<T>(val);
}

size_t table_bytes(const ctr_helical_param* p)
{
    return sizeof(HeliHeader) + sizeof(HeliChan) * p->ns + sizeof(HeliSlice) * p->nz;
}

int check_param(const ctr_helical_param* p)
{
    if (!p) return fail(CTR_ERR_INVALID_ARG, "null helical parameters");
    if (p->ns < 1 || p->nt < 1 || p->na < 1 || p->view_per_rot < 1 || p->nz < 1)
        return fail(CTR_ERR_INVALID_ARG, "empty helical geometry");
    const double f[] = {p->ds, p->offset_s, p->offset_t, p->orbit, p->couch_begin, p->couch_mov,
                        p->dz, p->z0, p->thickness, p->dso, p->dsd};
    for (double v : f)
        if (!std::isfinite(v)) return fail(CTR_ERR_INVALID_ARG, "non-finite helical parameter");
    if (p->couch_mov == 0.0 || p->orbit == 0.0 || p->dso == 0.0 || p->dsd == 0.0 || p->ds == 0.0)
        return fail(CTR_ERR_INVALID_ARG, "couch_mov, orbit, ds, dso and dsd must be non-zero");
    if (p->view_per_rot > 65535u) return fail(CTR_ERR_UNSUPPORTED, "view_per_rot > 65535");
    return CTR_OK;
}

template <typename T>
int helical_run(int method, const ctr_helical_param* p, const T* in, T* out, const void* table, unsigned* status,
                int batch, cudaStream_t stream)
{
    int st = check_param(p);
    if (st) return st;
    if (bad_ptr(in) || bad_ptr(out) || bad_ptr(table) || bad_ptr(status))
        return fail(CTR_ERR_INVALID_ARG, "null pointer");
    if ((st = check_common(batch))) return st;
    if (static_cast<unsigned long long>(p->nz) * batch > 65535ull)
        return fail(CTR_ERR_UNSUPPORTED, "nz * batch > 65535");
    HeliGeo g;
    g.ns = p->ns;
    g.nt = p->nt;
    g.na = p->na;
    g.vpr = p->view_per_rot;
    g.nz = p->nz;
    g.center_t = static_cast<double>(p->nt - 1) / 2.0 + p->offset_t;
    g.couch_begin = p->couch_begin;
    g.couch_mov = p->couch_mov;
    g.half_th = p->thickness / 2.0;
    g.dso = p->dso;
    g.dsd = p->dsd;
    g.nt_d = static_cast<double>(p->nt);
    g.ns_last = static_cast<double>(p->ns - 1);
    g.in_item = static_cast<size_t>(p->na) * p->nt * p->ns;
    g.out_item = static_cast<size_t>(p->nz) * p->view_per_rot * p->ns;
    const dim3 grid(div_up(p->ns, kHeliThreads), p->view_per_rot, p->nz * batch);
    const HeliHeader* tab = static_cast<const HeliHeader*>(table);
    if (method == CTR_HELICAL_360)
        helical_kernel<T, CTR_HELICAL_360><<<grid, kHeliThreads, 0, stream>>>(in, out, tab, g, status);
    else
        helical_kernel<T, CTR_HELICAL_180><<<grid, kHeliThreads, 0, stream>>>(in, out, tab, g, status);
    return check_launch(method == CTR_HELICAL_360 ? "helical 360LI" : "helical 180LI");
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

size_t ctr_helical_interpolation_table_bytes(const ctr_helical_param* p)
{
    return p ? table_bytes(p) : 0;
}

int ctr_helical_interpolation_prep(const ctr_helical_param* p, int method, void* table, cudaStream_t stream)
{
    int st = check_param(p);
    if (st) return st;
    if (method != CTR_HELICAL_360 && method != CTR_HELICAL_180)
        return fail(CTR_ERR_INVALID_ARG, "helical method must be CTR_HELICAL_360 or CTR_HELICAL_180");
    if (bad_ptr(table)) return fail(CTR_ERR_INVALID_ARG, "null table");
    std::vector<unsigned char> host(table_bytes(p));
    HeliHeader* hdr = reinterpret_cast<HeliHeader*>(host.data());
    HeliChan* ch = reinterpret_cast<HeliChan*>(hdr + 1);
    HeliSlice* sl = reinterpret_cast<HeliSlice*>(ch + p->ns);
    *hdr = HeliHeader{method, p->ns, p->nz, p->view_per_rot};
    // per channel (src/helical_interpolation.cc:174-175, 196, 214)
    const double center_s = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    for (unsigned is = 0; is < p->ns; ++is) {
        const double s = (static_cast<double>(is) - center_s) * p->ds;
        const double gamma = s / p->dsd;
        ch[is].cg = std::cos(gamma);
        ch[is].dif = (kHeliPi - 2 * gamma) / p->orbit;
        ch[is].sc = center_s - s / p->ds;
        ch[is].pad = 0.0;
    }
    // per slice: the view range checks of src/helical_interpolation.cc:84-90 (360LI) and 160-166
    // (180LI); a failing slice is marked and reported by the kernel in its status word
    const int vpr = static_cast<int>(p->view_per_rot);
    double z = p->z0;
    for (unsigned iz = 0; iz < p->nz; ++iz, z += p->dz) {
        const double cv = std::round((z - p->couch_begin) / p->couch_mov);
        HeliSlice& s = sl[iz];
        s = HeliSlice{z, 0, 0, 0, 0, 0, 0};
        if (!(std::fabs(cv) < 1e9)) continue;  // far outside any scan: invalid
        s.center = static_cast<int>(cv);
        if (method == CTR_HELICAL_360) {
            s.lo = s.center - vpr;
            s.hi = s.center + vpr - 1;
        } else {
            s.lo = s.center - vpr / 2;
            s.hi = s.lo + vpr - 1;
        }
        if (s.lo < 0 || static_cast<unsigned>(s.hi) >= p->na) continue;
        s.valid = 1;
        s.first = method == CTR_HELICAL_360
                      ? (s.lo / vpr + 1) * vpr
                      : static_cast<int>(std::ceil(s.lo / static_cast<double>(p->view_per_rot)) * p->view_per_rot);
    }
    cudaError_t e = cudaMemcpyAsync(table, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
    // the host vector dies on return: wait for the staged copy to leave it
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    return e == cudaSuccess ? CTR_OK : fail(CTR_ERR_CUDA, "helical table: %s", cudaGetErrorString(e));
}

int ctr_helical_interpolation_360_f32(const ctr_helical_param* p, const float* in, float* out, const void* table,
                                      unsigned int* status, int batch, cudaStream_t stream)
{
    return helical_run<float>(CTR_HELICAL_360, p, in, out, table, status, batch, stream);
}
int ctr_helical_interpolation_360_f64(const ctr_helical_param* p, const double* in, double* out,
                                      const void* table, unsigned int* status, int batch, cudaStream_t stream)
{
    return helical_run<double>(CTR_HELICAL_360, p, in, out, table, status, batch, stream);
}
int ctr_helical_interpolation_180_f32(const ctr_helical_param* p, const float* in, float* out, const void* table,
                                      unsigned int* status, int batch, cudaStream_t stream)
{
    return helical_run<float>(CTR_HELICAL_180, p, in, out, table, status, batch, stream);
}
int ctr_helical_interpolation_180_f64(const ctr_helical_param* p, const double* in, double* out,
                                      const void* table, unsigned int* status, int batch, cudaStream_t stream)
{
    return helical_run<double>(CTR_HELICAL_180, p, in, out, table, status, batch, stream);
}

}  // extern "C"

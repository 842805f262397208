// Helical rebinning: 3-D helical sinograms to 2-D fan-beam sinograms, one per
// reconstructed slice, by 360LI or 180LI z interpolation (reference
// src/helical_interpolation.cc:80-370, include/helical_interpolation.h).
//
// The reference runs this on the CPU only.  Here one thread computes one
// output sample (slice, view, channel).  T=double runs the exact kernel: every
// operation is an FP64 intrinsic in the reference's order (__dadd_rn and
// friends, so nothing is contracted into an FMA), and the per-channel
// cos(gamma) and per-slice view ranges come from the host
// (ctr_helical_interpolation_prep) with the reference's own libm calls, so the
// output equals the reference's bit for bit.  T=float runs the FP32 fast path
// (helical_fast_f32): the same decisions as the reference (rows, usability,
// views) with FP32 sums, falling back to the exact computation per sample
// where an FP32 decision could differ; GB300's FP64 rate is 1/64 of its FP32
// rate, which made the exact kernel compute-bound at <1 % of HBM bandwidth.
//
// Layout: input [na][nt][ns] (view, detector row, channel), output
// [nz][view_per_rot][ns]; a block covers 128 consecutive channels of one
// (slice, view) row, so every row read is a coalesced channel run.
#include <cmath>
#include <type_traits>
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
    float ct_f, nt_f, hth_f, vprcm_f;  // FP32 fast path: center_t, nt, thickness / 2, vpr * couch_mov
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

// The reference's value of one output sample (slice s, output view iv,
// channel is), in FP64 and bit for bit: src/helical_interpolation.cc:93-149
// (360LI) and 169-248 (180LI).  ORs CTR_HELICAL_NO_ROWS / _OUTSIDE into *status.
template <typename T, int M>
__device__ double heli_exact(const T* __restrict__ in, const HeliGeo& g, const HeliSlice& s, const HeliChan& c,
                             unsigned iv, unsigned is, unsigned* status)
{
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
            if (c.sc < 0.0 || c.sc > g.ns_last) return vcur;  // mirrored channel off the detector
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
    if (ucur && ucor) return __ddiv_rn(__dsub_rn(__dmul_rn(zd, vcor), __dmul_rn(zd2, vcur)), __dsub_rn(zd, zd2));
    if (ucur) return vcur;
    if (ucor) return vcor;
    atomicOr(status, CTR_HELICAL_NO_ROWS);  // the reference throws "No row data available!"
    return 0.0;
}

// Table checks shared by both kernels: false (and nothing to do) for a table
// of another method or geometry, or for a slice the reference rejects.
template <int M>
__device__ __forceinline__ bool heli_slice_ok(const HeliHeader* tab, const HeliGeo& g, const HeliSlice& s,
                                              unsigned* status)
{
    if (tab->method != M || tab->ns != g.ns || tab->nz != g.nz || tab->vpr != g.vpr) {
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0)
            atomicOr(status, CTR_HELICAL_BAD_TABLE);
        return false;
    }
    if (!s.valid) {  // the reference throws before touching this slice
        if (threadIdx.x == 0 && blockIdx.x == 0 && blockIdx.y == 0) atomicOr(status + blockIdx.z, CTR_HELICAL_NO_VIEWS);
        return false;
    }
    return true;
}

template <int M>
__device__ __forceinline__ const HeliSlice* heli_slices(const HeliHeader* tab, const HeliGeo& g)
{
    return reinterpret_cast<const HeliSlice*>(reinterpret_cast<const HeliChan*>(tab + 1) + g.ns);
}

// The exact kernel (T=double, and T=float where the fast path's conditions do
// not hold): every sample through heli_exact.
template <typename T, int M>
__global__ void __launch_bounds__(kHeliThreads)
    helical_kernel(const T* __restrict__ in, T* __restrict__ out, const HeliHeader* __restrict__ tab, HeliGeo g,
                   unsigned* status)
{
    const unsigned iz = blockIdx.z % g.nz, b = blockIdx.z / g.nz;
    const HeliSlice s = heli_slices<M>(tab, g)[iz];
    if (!heli_slice_ok<M>(tab, g, s, status)) return;
    const unsigned is = blockIdx.x * kHeliThreads + threadIdx.x;
    if (is >= g.ns) return;
    const unsigned iv = blockIdx.y;
    const HeliChan c = reinterpret_cast<const HeliChan*>(tab + 1)[is];
    out[b * g.out_item + (static_cast<size_t>(iz) * g.vpr + iv) * g.ns + is] =
        static_cast<T>(heli_exact<T, M>(in + b * g.in_item, g, s, c, iv, is, status + blockIdx.z));
}

// ---- FP32 fast path (T = float) ---------------------------------------------
// The only discontinuous decisions of a sample are its row range (floor/ceil
// of the projected slab edges, usability) and, for 180LI, the complementary
// ray's integer view and wrap.  The fast path
//   * evaluates the slab edges in FP32 from per-(slice, view) quotients that
//     one thread of the block forms in FP64 with the reference's operations;
//     their FP32 error stays below 1e-4 rows, so wherever an edge lies more
//     than kEdgeGuard from an integer the FP32 decision is the reference's,
//     and any other sample is recomputed by heli_exact;
//   * takes the 180LI view offset from the host split dif = dif_i + f: with
//     f in [1e-6, 1 - 1e-6] (else the channel runs heli_exact) and views below
//     2^20, the reference's rounded cur - dif lies strictly inside
//     (cur - dif_i - 1, cur - dif_i), so its floor, ceil and wraps are integer
//     arithmetic here, and its interpolation weight is 1 - f to 1e-10;
//   * sums the rows and interpolates in FP32 (the reference: FP64), which keeps
//     every output within a few FP32 ulps of the reference's.

// An FP32 slab edge x is trusted when it lies farther than
// kEdgeGuard + (|x| + |center_t|) * kEdgeGuardRel from every integer: the FP32
// error of the edges is below 2e-5 rows + 4e-7 * (|x| + |center_t|).
constexpr float kEdgeGuard = 1.0f / 16384.0f;
constexpr float kEdgeGuardRel = 1.0f / 1048576.0f;

// Per-channel FP32 section of the table (after the slices).
struct HeliChanF {
    float g;      // cos(gamma) * dsd: rows per unit of (z_dif +- thickness/2) / dso
    float h;      // cos(gamma) * dsd / dso: rows per mm of z_dif
    float difcm;  // 180LI: dif * couch_mov, the complementary ray's z offset before wrapping
    float u;      // 180LI: 1 - frac(dif), the right view's weight
    float v;      // 180LI: sc - floor(sc), the right channel's weight
    int dif_i;    // 180LI: floor(dif)
    int cl, cr;   // 180LI: floor(sc), ceil(sc); cl = -1 when the mirrored channel is off the detector
    int exact;    // 180LI: frac(dif) within 1e-6 of 0 or 1: samples of this channel run heli_exact
    int pad;
};
static_assert(sizeof(HeliChanF) == 40, "table layout");

// One (slice, view) row of the table's last section, formed once per geometry
// by heli_rows_kernel with the reference's FP64 operations.
struct HeliRowF {
    double at_d[4];          // (z_dif +- thickness/2) / dso, exact: measured view top/bottom, paired view (360LI)
    double zrel;             // z - couch_begin
    float at, ab, at2, ab2;  // the same, rounded
    float zd, wcur, wcor;    // z_dif; 360LI: the z interpolation weights
    int cur, cor;
    int pad;
};
static_assert(sizeof(HeliRowF) == 80, "table layout");

template <int M>
__device__ __forceinline__ const HeliRowF* heli_rows_f(const HeliHeader* tab, const HeliGeo& g)
{
    const HeliChanF* cf = reinterpret_cast<const HeliChanF*>(heli_slices<M>(tab, g) + g.nz);
    return reinterpret_cast<const HeliRowF*>(cf + g.ns);
}

// The per-row section: one thread per (slice, view) of a valid slice.
template <int M>
__global__ void heli_rows_kernel(HeliHeader* tab, HeliGeo g)
{
    const unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= static_cast<unsigned long long>(g.nz) * g.vpr) return;
    const unsigned iz = static_cast<unsigned>(i / g.vpr), iv = static_cast<unsigned>(i % g.vpr);
    const HeliSlice s = heli_slices<M>(tab, g)[iz];
    HeliRowF row{};
    if (s.valid) {
        const double zrel = __dsub_rn(s.z, g.couch_begin);
        int cur = s.first + static_cast<int>(iv);
        if (M == CTR_HELICAL_180 && cur > s.hi) cur -= static_cast<int>(g.vpr);
        const double zd = __dsub_rn(zrel, __dmul_rn(static_cast<double>(cur), g.couch_mov));
        row.cur = cur;
        row.zrel = zrel;
        row.zd = static_cast<float>(zd);
        row.at_d[0] = __ddiv_rn(__dadd_rn(zd, g.half_th), g.dso);
        row.at_d[1] = __ddiv_rn(__dsub_rn(zd, g.half_th), g.dso);
        row.at = static_cast<float>(row.at_d[0]);
        row.ab = static_cast<float>(row.at_d[1]);
        if (M == CTR_HELICAL_360) {
            const int cor = cur >= s.center ? cur - static_cast<int>(g.vpr) : cur + static_cast<int>(g.vpr);
            const double zd2 = __dsub_rn(zrel, __dmul_rn(static_cast<double>(cor), g.couch_mov));
            row.cor = cor;
            row.at_d[2] = __ddiv_rn(__dadd_rn(zd2, g.half_th), g.dso);
            row.at_d[3] = __ddiv_rn(__dsub_rn(zd2, g.half_th), g.dso);
            row.at2 = static_cast<float>(row.at_d[2]);
            row.ab2 = static_cast<float>(row.at_d[3]);
            row.wcur = static_cast<float>(-zd2 / (zd - zd2));
            row.wcor = static_cast<float>(zd / (zd - zd2));
        }
    }
    const_cast<HeliRowF*>(heli_rows_f<M>(tab, g))[i] = row;
}

__device__ __forceinline__ bool near_int(float x, float ct)
{
    return fabsf(x - rintf(x)) < kEdgeGuard + (fabsf(x) + ct) * kEdgeGuardRel;
}

// An exact FP64 edge as an FP32 value with the same floor, ceil and order
// against every integer: the integer itself, or the midpoint of its cell.
__device__ __forceinline__ float snap_edge(double x)
{
    const double f = floor(x);
    return static_cast<float>(f == x ? x : f + 0.5);
}

// The reference's edge ct - (q * cos(gamma)) * dsd for an exact quotient q.
__device__ __forceinline__ float exact_edge(const HeliGeo& g, double q, double cg)
{
    return snap_edge(__dsub_rn(g.center_t, __dmul_rn(__dmul_rn(q, cg), g.dsd)));
}

// Rows [r0, r1) from FP32 slab edges already known to be away from integers.
__device__ __forceinline__ bool rows_f(float top, float bot, float nt, int& r0, int& r1)
{
    if (bot < 0.0f || top >= nt) return false;
    r0 = static_cast<int>(floorf(fmaxf(top, 0.0f)));
    r1 = static_cast<int>(ceilf(fminf(bot, nt)));
    return true;
}

__device__ __forceinline__ float mean_f(const float* __restrict__ col, unsigned ns, int r0, int r1)
{
    float acc = 0.0f;
    for (int r = r0; r < r1; ++r) acc += __ldg(col + static_cast<size_t>(r) * ns);
    return __fdividef(acc, static_cast<float>(r1 - r0));  // within 2 ulp; 0/0 stays NaN
}

__device__ __forceinline__ float at_f(const float* __restrict__ in, const HeliGeo& g, int view, int r, int c,
                                      bool& outside)
{
    if (view < 0 || static_cast<unsigned>(view) >= g.na) {
        outside = true;
        return 0.0f;
    }
    return __ldg(in + (static_cast<size_t>(view) * g.nt + r) * g.ns + c);
}

// One output sample of the fast path, written to *o.
template <int M>
__device__ __forceinline__ void heli_fast_one(const float* __restrict__ in, float* o, const HeliHeader* tab,
                                              const HeliGeo& g, const HeliSlice& s, const HeliRowF& row,
                                              const HeliChanF& cf, unsigned iv, unsigned is, unsigned* status)
{
    const float ct = g.ct_f, nt = g.nt_f;
    const size_t view_stride = static_cast<size_t>(g.nt) * g.ns;

    if (M == CTR_HELICAL_180 && cf.exact) {  // complementary view offset too close to an integer
        const HeliChan c = reinterpret_cast<const HeliChan*>(tab + 1)[is];
        *o = static_cast<float>(heli_exact<float, M>(in, g, s, c, iv, is, status));
        return;
    }
    const float cta = fabsf(ct);
    float top = ct - row.at * cf.g, bot = ct - row.ab * cf.g;
    if (near_int(top, cta) || near_int(bot, cta)) {  // rare: the reference's edges, exactly
        const double cg = reinterpret_cast<const HeliChan*>(tab + 1)[is].cg;
        top = exact_edge(g, row.at_d[0], cg);
        bot = exact_edge(g, row.at_d[1], cg);
    }
    float top2, bot2, zd2 = 0.0f;
    int k = 0;
    if (M == CTR_HELICAL_360) {
        top2 = ct - row.at2 * cf.g;
        bot2 = ct - row.ab2 * cf.g;
        if (near_int(top2, cta) || near_int(bot2, cta)) {
            const double cg = reinterpret_cast<const HeliChan*>(tab + 1)[is].cg;
            top2 = exact_edge(g, row.at_d[2], cg);
            bot2 = exact_edge(g, row.at_d[3], cg);
        }
    } else {
        // complementary view: k - f with k = cur - dif_i, wrapped into [lo, hi] as the reference wraps cv
        k = row.cur - cf.dif_i;
        int wrap = 0;
        if (k <= s.lo) { k += static_cast<int>(g.vpr); wrap += 1; }
        if (k > s.hi) { k -= static_cast<int>(g.vpr); wrap -= 1; }
        zd2 = row.zd + cf.difcm - static_cast<float>(wrap) * g.vprcm_f;
        const float hth = g.hth_f;
        top2 = ct - (zd2 + hth) * cf.h;
        bot2 = ct - (zd2 - hth) * cf.h;
        if (near_int(top2, cta) || near_int(bot2, cta)) {
            // the reference's complementary ray: cv = cur - dif wrapped, zd2 = zrel - cv * couch_mov
            const HeliChan c = reinterpret_cast<const HeliChan*>(tab + 1)[is];
            double cv = __dsub_rn(static_cast<double>(row.cur), c.dif);
            if (cv < static_cast<double>(s.lo)) cv = __dadd_rn(cv, static_cast<double>(g.vpr));
            if (cv > static_cast<double>(s.hi)) cv = __dsub_rn(cv, static_cast<double>(g.vpr));
            const double zdd = __dsub_rn(row.zrel, __dmul_rn(cv, g.couch_mov));
            top2 = exact_edge(g, __ddiv_rn(__dadd_rn(zdd, g.half_th), g.dso), c.cg);
            bot2 = exact_edge(g, __ddiv_rn(__dsub_rn(zdd, g.half_th), g.dso), c.cg);
        }
    }
    int r0 = 0, r1 = 0;
    float vcur = 0.0f, vcor = 0.0f;
    const bool ucur = rows_f(top, bot, nt, r0, r1);
    if (ucur) vcur = mean_f(in + row.cur * view_stride + is, g.ns, r0, r1);
    const bool ucor = rows_f(top2, bot2, nt, r0, r1);
    float val;
    if (M == CTR_HELICAL_360) {
        if (ucor) vcor = mean_f(in + row.cor * view_stride + is, g.ns, r0, r1);
        val = ucur && ucor ? row.wcor * vcor + row.wcur * vcur : (ucur ? vcur : vcor);
    } else {
        if (ucor) {
            if (cf.cl < 0) {  // mirrored channel off the detector: no interpolation
                *o = vcur;
                return;
            }
            const int vl = k - 1, vr = k;
            const float w = 1.0f - cf.v;
            float left = 0.0f, right = 0.0f;
            if (vl >= 0 && static_cast<unsigned>(vr) < g.na) {
                const float* pl = in + static_cast<size_t>(vl) * view_stride + static_cast<size_t>(r0) * g.ns;
                const float* pr = pl + view_stride;
                const int dc = cf.cr - cf.cl;
                for (int r = r0; r < r1; ++r, pl += g.ns, pr += g.ns) {
                    left += w * __ldg(pl + cf.cl) + cf.v * __ldg(pl + cf.cl + dc);
                    right += w * __ldg(pr + cf.cl) + cf.v * __ldg(pr + cf.cl + dc);
                }
            } else {  // a view outside the scan (only beside a slice whose first view is 0)
                bool outside = false;
                for (int r = r0; r < r1; ++r) {
                    left += w * at_f(in, g, vl, r, cf.cl, outside) + cf.v * at_f(in, g, vl, r, cf.cr, outside);
                    right += w * at_f(in, g, vr, r, cf.cl, outside) + cf.v * at_f(in, g, vr, r, cf.cr, outside);
                }
                if (outside) atomicOr(status, CTR_HELICAL_OUTSIDE);
            }
            vcor = __fdividef((1.0f - cf.u) * left + cf.u * right, static_cast<float>(r1 - r0));
        }
        val = ucur && ucor ? __fdividef(row.zd * vcor - zd2 * vcur, row.zd - zd2) : (ucur ? vcur : vcor);
    }
    if (!ucur && !ucor) {
        atomicOr(status, CTR_HELICAL_NO_ROWS);  // the reference throws "No row data available!"
        val = 0.0f;
    }
    *o = val;
}

// Views per block of the fast kernel: a block covers kHeliThreads channels of
// kHeliViews consecutive output views of one slice.
constexpr int kHeliViews = 16;

template <int M>
__global__ void __launch_bounds__(kHeliThreads, M == CTR_HELICAL_360 ? 8 : 6)
    helical_fast_f32(const float* __restrict__ in, float* __restrict__ out, const HeliHeader* __restrict__ tab,
                     HeliGeo g, unsigned* status)
{
    const unsigned iz = blockIdx.z % g.nz, b = blockIdx.z / g.nz;
    const HeliSlice s = heli_slices<M>(tab, g)[iz];
    if (!heli_slice_ok<M>(tab, g, s, status)) return;
    const unsigned is = blockIdx.x * kHeliThreads + threadIdx.x;
    if (is >= g.ns) return;
    in += b * g.in_item;
    status += blockIdx.z;
    const HeliChanF cf = reinterpret_cast<const HeliChanF*>(heli_slices<M>(tab, g) + g.nz)[is];
    const unsigned v0 = blockIdx.y * kHeliViews, v1 = min(v0 + kHeliViews, g.vpr);
    const HeliRowF* rows = heli_rows_f<M>(tab, g) + static_cast<size_t>(iz) * g.vpr;
    float* o = out + b * g.out_item + static_cast<size_t>(iz) * g.vpr * g.ns + is;
    for (unsigned iv = v0; iv < v1; ++iv)
        heli_fast_one<M>(in, o + static_cast<size_t>(iv) * g.ns, tab, g, s, rows[iv], cf, iv, is, status);
}

size_t table_bytes(const ctr_helical_param* p)
{
    return sizeof(HeliHeader) + sizeof(HeliChan) * p->ns + sizeof(HeliSlice) * p->nz + sizeof(HeliChanF) * p->ns +
           sizeof(HeliRowF) * static_cast<size_t>(p->nz) * p->view_per_rot;
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

HeliGeo make_geo(const ctr_helical_param* p)
{
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
    g.ct_f = static_cast<float>(g.center_t);
    g.nt_f = static_cast<float>(p->nt);
    g.hth_f = static_cast<float>(g.half_th);
    g.vprcm_f = static_cast<float>(p->view_per_rot * p->couch_mov);
    return g;
}

// Conditions of the FP32 fast path: a slab whose top edge lies above its
// bottom edge on every channel (thickness >= 0, dso and dsd > 0, |gamma| below
// pi/2), views and rows far inside the ranges its integer and FP32 arithmetic
// cover.  Elsewhere T=float runs the exact kernel.
bool fast_ok(const ctr_helical_param* p)
{
    const double center_s = static_cast<double>(p->ns - 1) / 2.0 + p->offset_s;
    const double gmax = std::fmax(std::fabs((0.0 - center_s) * p->ds / p->dsd),
                                  std::fabs((static_cast<double>(p->ns - 1) - center_s) * p->ds / p->dsd));
    return p->thickness >= 0.0 && p->dso > 0.0 && p->dsd > 0.0 && gmax < kHeliPi / 2 - 1e-3 &&
           p->na < (1u << 20) && p->nt < (1u << 15) && std::fabs(p->view_per_rot * p->couch_mov) < 1e4;
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
    const HeliGeo g = make_geo(p);
    const dim3 grid(div_up(p->ns, kHeliThreads), p->view_per_rot, p->nz * batch);
    const HeliHeader* tab = static_cast<const HeliHeader*>(table);
    if (std::is_same<T, float>::value && fast_ok(p)) {
        const float* fin = reinterpret_cast<const float*>(in);
        float* fout = reinterpret_cast<float*>(out);
        const dim3 grid(div_up(p->ns, kHeliThreads), div_up(p->view_per_rot, kHeliViews), p->nz * batch);
        if (method == CTR_HELICAL_360)
            helical_fast_f32<CTR_HELICAL_360><<<grid, kHeliThreads, 0, stream>>>(fin, fout, tab, g, status);
        else
            helical_fast_f32<CTR_HELICAL_180><<<grid, kHeliThreads, 0, stream>>>(fin, fout, tab, g, status);
        return check_launch(method == CTR_HELICAL_360 ? "helical 360LI (FP32)" : "helical 180LI (FP32)");
    }
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
    const size_t row_bytes = sizeof(HeliRowF) * static_cast<size_t>(p->nz) * p->view_per_rot;
    std::vector<unsigned char> host(table_bytes(p) - row_bytes);  // the rows are formed on the device
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
    // the FP32 fast path's per-channel section (from the same FP64 values)
    HeliChanF* cf = reinterpret_cast<HeliChanF*>(sl + p->nz);
    for (unsigned is = 0; is < p->ns; ++is) {
        const HeliChan& c = ch[is];
        HeliChanF& f = cf[is];
        f = HeliChanF{};
        f.g = static_cast<float>(c.cg * p->dsd);
        f.h = static_cast<float>(c.cg * p->dsd / p->dso);
        f.difcm = static_cast<float>(c.dif * p->couch_mov);
        const bool finite = std::fabs(c.dif) < static_cast<double>(1 << 20);
        const double di = finite ? std::floor(c.dif) : 0.0, fr = c.dif - di;
        f.dif_i = static_cast<int>(di);
        f.u = static_cast<float>(1.0 - fr);
        f.exact = (!finite || fr < 1e-6 || fr > 1.0 - 1e-6) ? 1 : 0;
        if (c.sc < 0.0 || c.sc > static_cast<double>(p->ns - 1)) {
            f.cl = f.cr = -1;
        } else {
            f.cl = static_cast<int>(std::floor(c.sc));
            f.cr = static_cast<int>(std::ceil(c.sc));
            f.v = static_cast<float>(c.sc - f.cl);
        }
    }
    cudaError_t e = cudaMemcpyAsync(table, host.data(), host.size(), cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) {
        const HeliGeo g = make_geo(p);
        const unsigned long long rows = static_cast<unsigned long long>(p->nz) * p->view_per_rot;
        if (rows > 65535ull * 65535ull) return fail(CTR_ERR_UNSUPPORTED, "nz * view_per_rot too large");
        HeliHeader* tab = static_cast<HeliHeader*>(table);
        if (method == CTR_HELICAL_360)
            heli_rows_kernel<CTR_HELICAL_360><<<div_up(rows, 256), 256, 0, stream>>>(tab, g);
        else
            heli_rows_kernel<CTR_HELICAL_180><<<div_up(rows, 256), 256, 0, stream>>>(tab, g);
        e = cudaGetLastError();
    }
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

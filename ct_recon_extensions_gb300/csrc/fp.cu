// Parallel-beam ray-driven forward projection and its adjoint (reference
// src/fp_par_2d.cc:210-391).
//
// Views whose rays run closer to the y axis (usex) march image rows and
// interpolate along x; the others march columns and interpolate along y.  A
// sample is included iff its fractional index lies in [0, n-1], the
// reference's CPU rule (src/fp_par_2d.cc:237,259); the ray sum is scaled by
// dy/|cos| or dx/|sin|.
//
// FP32 forward: a persistent-style pipeline streams the image (and a
// transposed copy for column-marching views) through shared memory in bands of
// rows with TMA bulk copies; each lane keeps a few rays in registers.  Each
// ray's sample range is decided once, in integer arithmetic with the
// reference's FP64 rule taken over at ties (fp_setup.cuh); positions are 32.32
// fixed point, so a sample costs one 64-bit add, two shared loads, the
// fraction and two FP32 operations.
//
// FP32 adjoint: one thread per pixel gathers, for every view, the channels of
// its footprint with the triangle weights of the reference's grad
// (src/fp_par_2d.cc:339-383), channel positions in 32.32 fixed point from the
// caller's grad-prep table.  The channel range is clamped to the detector
// (the reference reads without a bounds check there).  No atomics.
//
// FP64 kernels follow the reference's arithmetic (one thread per ray / pixel).
#include <algorithm>
#include <climits>
#include <memory>
#include <numeric>

#include "ctr_async.cuh"
#include "ctr_common.cuh"
#include "fp_setup.cuh"

namespace ctr {
namespace {

// ---- FP32 forward: image bands in shared memory, fixed-point sample positions

constexpr int kFpThreads = 512;
constexpr int kFpMaxRays = 8;  // rays per thread
// 2^32: the adjoint's channel positions are 32.32 fixed point.
constexpr double kTwo32 = 4294967296.0;

struct FpConst {
    int ns, na, nx, ny;
    int views;  // views per CTA
    int band;   // staged lines per band
    double dx, dy;
    size_t img_stride, proj_stride;
};

__device__ __forceinline__ float frac_of(long long X)
{
    return __uint_as_float(0x3F800000u | (static_cast<unsigned>(X) >> 9)) - 1.0f;
}

// 1 + frac(X) on the FMA pipe: the fraction's top 23 bits as a mantissa in
// one integer multiply-add, (lo * 2^23) >> 32 plus the bits of 1.0.  `m` (2^23)
// and `one` (0x3F800000) are run-time registers (see fpx_regs), so the multiply
// is not turned back into a shift on the half-rate integer ALU pipe, which the
// 64-bit position step and the address already load.
__device__ __forceinline__ float one_plus_frac(long long X, unsigned m, unsigned one)
{
    unsigned b;
    asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(b) : "r"(static_cast<unsigned>(X)), "r"(m), "r"(one));
    return __uint_as_float(b);
}

// Packed FP32 pairs: __fadd2_rn / __ffma2_rn (Blackwell FADD2 / FFMA2, two
// IEEE round-to-nearest operations in one instruction, independent halves).
// A difference is an FMA with -1 (exact negation, one rounding: the same as
// a subtraction).
__device__ __forceinline__ float2 f2_sub(float2 a, float2 b)
{
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}

// A CTA projects `views` consecutive views (all channels).  Rays of row-marching
// views (usex) and of column-marching views are run in separate passes; each
// pass stages the image in bands of `band` rows (or columns, stored transposed)
// that all rays of the pass read from shared memory.
__global__ void __launch_bounds__(kFpThreads)
    fp_band_f32(const float* __restrict__ img, float* __restrict__ proj,
                const double* __restrict__ sincos, const double* __restrict__ bo,
                const int* __restrict__ usex, const FpConst c)
{
    extern __shared__ float band[];  // [band][len + 1]
    const int v0 = blockIdx.x * c.views;
    const int nv = min(c.views, c.na - v0);
    const int nrays = nv * c.ns;
    const float* I = img + blockIdx.y * c.img_stride;

    long long X[kFpMaxRays], S[kFpMaxRays];
    int k0[kFpMaxRays], k1[kFpMaxRays], cls[kFpMaxRays];
    float sum[kFpMaxRays];
    bool has_cls[2] = {false, false};
#pragma unroll
    for (int j = 0; j < kFpMaxRays; ++j) {
        const int r = threadIdx.x + j * kFpThreads;
        sum[j] = 0.0f;
        cls[j] = -1;
        X[j] = 0;
        S[j] = 0;
        k0[j] = 0;
        k1[j] = -1;
        if (r < nrays) {
            const int ia = v0 + r / c.ns;
            const size_t ray = static_cast<size_t>(v0) * c.ns + r;
            const int ux = usex[ia] != 0;
            const double begin = bo[2 * ray], step = bo[2 * ray + 1];
            if (!ray_fixed(begin, step, c.nx, &X[j], &S[j], &k0[j], &k1[j]))
                ray_fp64(begin, step, c.nx, &X[j], &S[j], &k0[j], &k1[j]);
            cls[j] = ux ? 0 : 1;
            has_cls[cls[j]] = true;
        }
    }
    for (int pass = 0; pass < 2; ++pass) {
        if (!__syncthreads_or(has_cls[pass])) continue;
        const int n = pass == 0 ? c.ny : c.nx;    // samples along the ray
        const int len = pass == 0 ? c.nx : c.ny;  // staged line length
        const int ld = len + 1;                   // zero pad after each line
        for (int b0 = 0; b0 < n; b0 += c.band) {
            const int nb = min(c.band, n - b0);
            if (pass == 0) {
                for (int idx = threadIdx.x; idx < nb * ld; idx += kFpThreads) {
                    const int i = idx / ld, t = idx - i * ld;
                    band[idx] = t < len ? __ldg(I + static_cast<size_t>(b0 + i) * c.nx + t) : 0.0f;
                }
            } else {
                // column band: read rows of nb consecutive pixels, store transposed
                for (int idx = threadIdx.x; idx < nb * ld; idx += kFpThreads) {
                    const int t = idx / nb, i = idx - t * nb;
                    band[i * ld + t] = t < len ? __ldg(I + static_cast<size_t>(t) * c.nx + b0 + i) : 0.0f;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kFpMaxRays; ++j) {
                if (cls[j] != pass) continue;
                const int ka = max(k0[j], b0), kb = min(k1[j], b0 + nb - 1);
                if (ka > kb) continue;
                long long x = X[j] + static_cast<long long>(ka) * S[j];
                const float* line = band + (ka - b0) * ld;
                float acc = 0.0f;  // this band's partial sum (blocked summation)
                for (int k = ka; k <= kb; ++k, line += ld, x += S[j]) {
                    const int i1 = static_cast<int>(x >> 32);
                    const float u = frac_of(x);
                    const float p0 = line[i1], p1 = line[i1 + 1];
                    acc = fmaf(u, p1 - p0, acc + p0);
                }
                sum[j] += acc;
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int j = 0; j < kFpMaxRays; ++j) {
        const int r = threadIdx.x + j * kFpThreads;
        if (r < nrays) {
            const int ia = v0 + r / c.ns;
            const double dw = cls[j] == 0 ? fabs(c.dy / sincos[2 * ia + 1]) : fabs(c.dx / sincos[2 * ia]);
            proj[blockIdx.y * c.proj_stride + static_cast<size_t>(v0) * c.ns + r] =
                static_cast<float>(sum[j] * dw);
        }
    }
}

// ---- FP32 forward: ray set-up kernel + one pipelined pass over image bands ----
//
// fpx_setup decides every ray once: its sample range and 32.32 fixed-point
// line (fp_setup.cuh), written to a per-call table; block 0 also lists the
// views of each marching class and cuts the slots of each class among the
// projector's CTAs.  fp_proj_f32 then streams, per CTA, the image (row-marching
// views, usex) or its transposed copy (column-marching views) once through
// shared memory in bands of rows, so every ray marches rows of the staged
// array and every CTA serves one class.
//
// Rays are grouped in "slots" of 4 consecutive views of one class x 8
// consecutive channels, one ray per lane (lane = 8*view + channel), so a
// warp's 32 samples of one row fall within a few pixels of each other.  Slots
// are ordered view quad by view quad, and within a quad the channel octets in
// a strided order (slot_octet).  Each class gets CTAs (one an SM) in
// proportion to its views, and the G CTAs of a class take its slots in turn
// (CTA i: slots i, i + G, ...), so each CTA holds long central and short edge
// rays of views across the class's whole angular range; a CTA deals its
// slots, sorted by their exact sample counts, to its warps in snake order.  A
// round holds up to kFpxRound slots (one more round streams the image again;
// rare).
//
// Pipeline: a producer lane copies band t (one contiguous range of the staged
// row-major array, one TMA bulk copy) into stage t % 3 once every consumer
// warp has released that stage, so warps drift up to two bands apart instead
// of meeting at a CTA barrier per band.  One CTA of 19 consumer warps (6
// slots each) and a producer warp runs on each SM, with three 64 KB stages.
// Within a band a sample costs one 64-bit add, the address, two shared loads,
// the fraction (one integer multiply-add on the FMA pipe) and two FP32
// operations, packed two rows to an instruction: the position's high word
// indexes the stage directly (S2 = S + n * 2^32 steps one row down).  A band
// is walked in chunks of CH rows, slot by slot, with warp-uniform decisions: a slot none of whose rays
// reaches the band is skipped, a chunk every ray of the slot covers runs
// unrolled without tests, and only chunks where some ray starts or ends test
// each row against the lane's range.
//
// Ties: a ray whose end sample lies within a hair of the image border (where
// the fixed-point rule might differ from the reference's accumulated FP64
// one) streams only its certain samples; the set-up decides its few border
// samples by the reference's accumulation (acc_advance) and the ray's lane
// adds the ones found inside, read from global memory, before writing.
constexpr int kFpxWarps = 19;                        // consumer warps (one CTA an SM)
constexpr int kFpxThreads = (kFpxWarps + 1) * 32;    // + one producer warp
constexpr int kFpxSlots = 6;                         // ray slots per consumer lane and round
constexpr int kFpxRound = kFpxWarps * kFpxSlots;     // slots per round
constexpr int kFpxStages = 3;
constexpr int kFpxStageFloats = 16384;               // nominal stage: 64 KB
constexpr int kFpxEmpty = 0x7FFF;                    // ray code of a ray with no sample (k0 > k1)
constexpr unsigned kFpxExc = 1u << 31;               // ray code flag: own line and tie in the per-ray tables
constexpr long long kFpxLineTol = 256;               // |model - own line start| allowed, units of 2^-32 px
constexpr int kFpxMaxTies = 8192;                    // tie rays per call
constexpr int kFpxSetupThreads = 256;

struct FpxConst {
    int ns, na, n;
    int octets;            // channel octets per view quad
    int stride;            // octet order within a quad: octet = rank * stride mod octets
    int quads;             // view quads without class padding: ceil(na / 4)
    int ctas;              // CTAs per item
    int band, nbands;      // image rows per stage; stages
    int stage_floats;      // floats per stage (>= band*n + 8, multiple of 32)
    long long total;       // elements of one staged array (batch * n * n)
    long long total4;      // total rounded down to 4
    size_t proj_stride;
    float dx, dy;
    int sms;               // SMs of the device
    unsigned frac_mul;     // 2^23 (one_plus_frac)
    unsigned frac_one;     // 0x3F800000, the bits of 1.0f (one_plus_frac)
};

// A view's model line: sample 0 of channel is at x0 + is*d2, step S (32.32),
// with FP32 estimates of where channel is crosses the image's ends,
// t0 = a + is*b and t1 = t0 + c samples.
struct FpxLine {
    long long x0, d2, S;
    float a, b, c;
    int pad;
};

// Global tie entry (a ray the fixed-point rule could not settle).
struct FpxTie {
    int namb;
    unsigned in;  // bit a: amb[a] is inside by the reference's accumulated rule
    int amb[4];   // ambiguous samples next to the certain range
};

// The per-call tables (scratch) written by fpx_setup.  The projector derives
// a ray's line and sample range from its view's model line (24 bytes a view)
// and reads one exception bit; only flagged rays (ties, the FP64 path, a line
// or range off the view's model) read their code, X0, S and tie.
struct FpxRays {
    float* vw;       // [na] ray weight of the view: dy/|cos| (row-marching) or dx/|sin|
    FpxLine* line;   // [na] the views' model lines
    unsigned* exc;   // [na * octets bits, in words] bit 8*(ia*octets + octet) + c: channel
                     // 8*octet + c of view ia is flagged kFpxExc (zeroed before fpx_setup)
    long long* X0;   // [na*ns] 32.32 position of sample 0
    long long* S;    // [na*ns] 32.32 step
    int* code;       // [na*ns] k0 | k1 << 15 | class << 30 | kFpxExc (empty: k0 > k1)
    int* tie;        // [na*ns] index into ties, or -1
    int* views;      // [4 * (quads + 2)] views of class 0, then of class 1, -1 padded to quads
    int* cuts;       // [3]: CTAs of class 0, slots of class 0, slots of class 1
    FpxTie* ties;    // [kFpxMaxTies]
    int* nties;      // count (zeroed before fpx_setup)
};

// Bytes of the exception bitmap: one byte per (view, channel octet).
__host__ __device__ inline size_t fpx_exc_bytes(long long rays, int na)
{
    const size_t octets = na > 0 ? (static_cast<size_t>(rays / na) + 7) / 8 : 0;
    return (static_cast<size_t>(na) * octets + 255) & ~static_cast<size_t>(255);
}

__host__ __device__ inline size_t fpx_table_bytes(long long rays, int na, int ctas)
{
    const size_t r = static_cast<size_t>(rays);
    const size_t views = 4 * (static_cast<size_t>(na) / 4 + 3);
    const size_t vw = (static_cast<size_t>(na) * 4 + 255) & ~static_cast<size_t>(255);
    const size_t line = (static_cast<size_t>(na) * sizeof(FpxLine) + 255) & ~static_cast<size_t>(255);
    return vw + line + fpx_exc_bytes(rays, na) + ((r * 24 + views * 4 + (static_cast<size_t>(ctas) + 2) * 4 + 63) & ~static_cast<size_t>(63)) +
           64 + static_cast<size_t>(kFpxMaxTies) * sizeof(FpxTie);
}

// Channel octet of the slot with rank `r` within its view quad.  Ranks run
// through the octets with a stride near 0.618 * octets (coprime), so a CTA's
// contiguous range of slots mixes central rays (long) and edge rays (short or
// empty).
__device__ __forceinline__ int slot_octet(unsigned r, const FpxConst& c)
{
    return static_cast<int>((r * static_cast<unsigned>(c.stride)) % static_cast<unsigned>(c.octets));
}

// The ray of slot q on lane `lane`: view ia (-1: padding) and channel is.
__device__ __forceinline__ void slot_ray(unsigned q, int lane, const FpxConst& c, const int* views,
                                         int* ia, int* is)
{
    const unsigned quad = q / static_cast<unsigned>(c.octets);
    *ia = views[quad * 4 + (lane >> 3)];
    *is = slot_octet(q - quad * static_cast<unsigned>(c.octets), c) * 8 + (lane & 7);
}

// imgT[b][x][y] = img[b][y][x] for the 32 x 32 tile `tb` (tiles of every
// item in a row); t is 32 x 33 floats of shared memory.
__device__ __forceinline__ void fpx_transpose_tile(const float* __restrict__ img, float* __restrict__ imgT,
                                                   int n, int tb, float (*t)[33])
{
    const int tid = threadIdx.x;
    const int tiles = (n + 31) / 32;
    const int item = tb / (tiles * tiles), tt = tb - item * tiles * tiles;
    const int x0 = (tt % tiles) * 32, y0 = (tt / tiles) * 32;
    const int tx = tid & 31, ty = tid >> 5;
    const size_t off = static_cast<size_t>(item) * n * n;
    for (int rr = ty; rr < 32; rr += kFpxSetupThreads / 32) {
        const int y = y0 + rr, x = x0 + tx;
        if (x < n && y < n) t[rr][tx] = img[off + static_cast<size_t>(y) * n + x];
    }
    __syncthreads();
    for (int rr = ty; rr < 32; rr += kFpxSetupThreads / 32) {
        const int x = x0 + rr, y = y0 + tx;
        if (x < n && y < n) imgT[off + static_cast<size_t>(x) * n + y] = t[tx][rr];
    }
}

// The transposed copy alone (the plan's calls: its ray tables already exist).
__global__ void __launch_bounds__(kFpxSetupThreads)
    fpx_transpose(const float* __restrict__ img, float* __restrict__ imgT, int n)
{
    __shared__ float t[32][33];
    fpx_transpose_tile(img, imgT, n, static_cast<int>(blockIdx.x), t);
}

// A begin the view model may take (|v| < 2^20 px, fix32's exact range; NaN
// and infinities fail).
__device__ __forceinline__ bool line_ok(double v) { return fabs(v) < 1048576.0; }

// a / b rounded to nearest (ties away from zero), b > 0.
__device__ __forceinline__ long long round_div(long long a, long long b)
{
    return a >= 0 ? (a + b / 2) / b : -((-a + b / 2) / b);
}

// The FP32 constants of a view's crossing estimates (view_range): channel
// is crosses 0 at sample -(x0 + is*d2)/S and n-1 at ((n-1)*2^32 - x0 - is*d2)/S.
__device__ __forceinline__ FpxLine view_line(long long x0, long long d2, long long S, int n)
{
    FpxLine l{x0, d2, S, 0.0f, 0.0f, 0.0f, 0};
    if (S != 0) {
        const float s = fix_to_float(S);
        l.a = -fix_to_float(x0) / s;
        l.b = -fix_to_float(d2) / s;
        l.c = static_cast<float>(n - 1) / s;
    }
    return l;
}

// The sample range [*k0, *k1] (empty: k0 = kFpxEmpty, k1 = 0) of channel is
// of a view's model line, X(k) = x0 + is*d2 + k*S inside [0, (n-1)*2^32]: the
// FP32 crossing estimates settled by up to three exact steps at each end.  A
// ray keeps the range derived this way only where the set-up found it equal
// to the exact one (every other ray is flagged and reads its own code).
__device__ __forceinline__ void view_range(const FpxLine& l, int is, int n, int* k0o, int* k1o)
{
    const long long L = static_cast<long long>(n - 1) << 32;
    const long long X0 = l.x0 + static_cast<long long>(is) * l.d2, S = l.S;
    auto inside = [&](int k) {
        const long long x = X0 + static_cast<long long>(k) * S;
        return x >= 0 && x <= L;
    };
    int k0, k1;
    if (S == 0) {
        k0 = 0;
        k1 = inside(0) ? n - 1 : -1;
    } else {
        const float t0 = fmaf(static_cast<float>(is), l.b, l.a), t1 = t0 + l.c;
        const float lim = static_cast<float>(n + 2);
        const float ta = fminf(fmaxf(fminf(t0, t1), -2.0f), lim);
        const float tb = fminf(fmaxf(fmaxf(t0, t1), -2.0f), lim);
        k0 = max(0, static_cast<int>(ceilf(ta)));
        k1 = min(n - 1, static_cast<int>(floorf(tb)));
        for (int it = 0; it < 3 && k0 > 0 && inside(k0 - 1); ++it) --k0;
        for (int it = 0; it < 3 && k0 <= k1 && !inside(k0); ++it) ++k0;
        for (int it = 0; it < 3 && k1 < n - 1 && inside(k1 + 1); ++it) ++k1;
        for (int it = 0; it < 3 && k1 >= k0 && !inside(k1); ++it) --k1;
    }
    if (k0 > k1) {
        k0 = kFpxEmpty;
        k1 = 0;
    }
    *k0o = k0;
    *k1o = k1;
}

// ---- set-up kernel: every ray once; block 0 the class lists, CTA cut and view
// weights.  Blocks from `setup_blocks` on transpose the images instead (32 x 32
// tiles): the two jobs are independent, and the transpose blocks fill the SMs
// left idle while the few tie rays of the set-up walk the reference's
// accumulation.
__global__ void __launch_bounds__(kFpxSetupThreads)
    fpx_setup(const double* __restrict__ bo, const int* __restrict__ usex, const double* __restrict__ sincos,
              const FpxConst c, const FpxRays r, int setup_blocks, const float* __restrict__ img,
              float* __restrict__ imgT)
{
    __shared__ int s_chunk[2049];  // block 0: row-marching views before each chunk of 32
    const int tid = threadIdx.x;
    if (static_cast<int>(blockIdx.x) >= setup_blocks) {
        fpx_transpose_tile(img, imgT, c.n, static_cast<int>(blockIdx.x) - setup_blocks,
                           reinterpret_cast<float (*)[33]>(s_chunk));
        return;
    }
    if (blockIdx.x == 0) {
        // ray weight of each view: the reference's dy/|cos| or dx/|sin|, in FP32
        for (int ia = tid; ia < c.na; ia += kFpxSetupThreads)
            r.vw[ia] = usex[ia] != 0 ? c.dy / fabsf(dbl2flt(sincos[2 * ia + 1]))
                                     : c.dx / fabsf(dbl2flt(sincos[2 * ia]));
        // class lists with warp ballots over chunks of 32 views: row-marching
        // views (usex) first, then column-marching ones, each padded to quads
        constexpr int kWarps = kFpxSetupThreads / 32;
        const int warp = tid >> 5, lane = tid & 31;
        const int nch = (c.na + 31) / 32;
        for (int ch = warp; ch < nch; ch += kWarps) {
            const int v = ch * 32 + lane;
            const unsigned b = __ballot_sync(0xffffffffu, v < c.na && usex[v] != 0);
            if (lane == 0) s_chunk[ch + 1] = __popc(b);
        }
        __syncthreads();
        if (warp == 0) {  // running count of row-marching views before each chunk
            int carry = 0;
            if (lane == 0) s_chunk[0] = 0;
            for (int base = 0; base < nch; base += 32) {
                int x = base + lane < nch ? s_chunk[base + lane + 1] : 0;
                for (int off = 1; off < 32; off <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, x, off);
                    if (lane >= off) x += y;
                }
                if (base + lane < nch) s_chunk[base + lane + 1] = carry + x;
                carry += __shfl_sync(0xffffffffu, x, 31);
            }
        }
        __syncthreads();
        const int N0 = s_chunk[nch], N1 = c.na - N0;
        const int Q0 = (N0 + 3) / 4, Q1 = (N1 + 3) / 4, Qt = Q0 + Q1;
        for (int ch = warp; ch < nch; ch += kWarps) {
            const int v = ch * 32 + lane;
            const bool row = v < c.na && usex[v] != 0;
            const unsigned below = __ballot_sync(0xffffffffu, row) & ((1u << lane) - 1u);
            const int o0 = s_chunk[ch] + __popc(below);                        // row views before v
            const int o1 = (ch * 32 - s_chunk[ch]) + (lane - __popc(below));  // column views before v
            if (v < c.na) r.views[row ? o0 : 4 * Q0 + o1] = v;
        }
        for (int i = N0 + tid; i < 4 * Q0; i += kFpxSetupThreads) r.views[i] = -1;
        for (int i = 4 * Q0 + N1 + tid; i < 4 * Qt; i += kFpxSetupThreads) r.views[i] = -1;
        // CTAs per class in proportion to its views; a class's CTAs take its
        // slots in turn (CTA i of G: slots i, i + G, i + 2G, ...), so every CTA
        // holds views of the class's whole angular range (the samples of a
        // view scale with |cos| or |sin| of its angle) and all CTAs carry about
        // the same work
        int G0 = 0;
        if (N0 > 0) G0 = N1 > 0 ? static_cast<int>(rintf(static_cast<float>(c.ctas) * N0 / c.na)) : c.ctas;
        if (N0 > 0 && N1 > 0) G0 = max(1, min(c.ctas - 1, G0));
        if (tid == 0) {
            r.cuts[0] = G0;
            r.cuts[1] = Q0 * c.octets;  // slots of class 0 (class 1 starts there)
            r.cuts[2] = Q1 * c.octets;  // slots of class 1
        }
    }
    const int rays = c.na * c.ns;
    for (int ray = blockIdx.x * kFpxSetupThreads + tid; ray < rays; ray += setup_blocks * kFpxSetupThreads) {
        const int ia = ray / c.ns;
        const double begin = bo[2 * static_cast<size_t>(ray)], step = bo[2 * static_cast<size_t>(ray) + 1];
        long long X0 = 0, S = 0;
        int k0, k1, tie = -1;
        const bool plain = ray_fixed(begin, step, c.n, &X0, &S, &k0, &k1);
        if (!plain) {
            int amb[4], namb = 0;
            bool done = false;
            if (ray_split(begin, step, c.n, &X0, &S, &k0, &k1, amb, &namb)) {
                const int e = atomicAdd(r.nties, 1);
                if (e < kFpxMaxTies) {
                    // the reference's decisions for the ambiguous samples, walked in order
                    for (int a = 1; a < namb; ++a)
                        for (int b = a; b > 0 && amb[b] < amb[b - 1]; --b) {
                            const int tmp = amb[b];
                            amb[b] = amb[b - 1];
                            amb[b - 1] = tmp;
                        }
                    AccWalk w{begin, 0};
                    unsigned in = 0u;
                    for (int a = 0; a < namb; ++a) {
                        acc_advance(&w, step, amb[a]);
                        if (w.x >= 0.0 && w.x <= static_cast<double>(c.n - 1)) in |= 1u << a;
                    }
                    FpxTie& t = r.ties[e];
                    t.namb = namb;
                    t.in = in;
                    for (int a = 0; a < 4; ++a) t.amb[a] = a < namb ? amb[a] : 0;
                    tie = e;
                    done = true;
                }
            }
            if (!done) ray_fp64(begin, step, c.n, &X0, &S, &k0, &k1);
        }
        // the view's linear model, from its first and last channels (every
        // ray of the view computes it alike): x0 + is * d2, step Sv
        const int is = ray - ia * c.ns;
        const double* bv = bo + 2 * static_cast<size_t>(ia) * c.ns;
        const double bl = bv[2 * static_cast<size_t>(c.ns - 1)];
        const bool model = line_ok(bv[0]) && line_ok(bl) && fabs(bv[1]) < 4.0;
        const long long x0 = model ? fix32(bv[0]) : 0, Sv = model ? fix32(bv[1]) : 0;
        const long long d2 = model && c.ns > 1 ? round_div(fix32(bl) - x0, c.ns - 1) : 0;
        const FpxLine vl = view_line(x0, d2, Sv, c.n);
        if (is == 0) r.line[ia] = vl;
        const long long dev = x0 + static_cast<long long>(is) * d2 - X0;
        bool own = !model || tie >= 0 || !plain || S != Sv || dev > kFpxLineTol || dev < -kFpxLineTol;
        if (!own) {
            // the projector derives the range from the model line: keep it
            // only where that gives the exact range
            int m0, m1;
            view_range(vl, is, c.n, &m0, &m1);
            own = k0 <= k1 ? (m0 != k0 || m1 != k1) : m0 <= m1;
        }
        if (own) {
            const long long bit = (static_cast<long long>(ia) * c.octets + (is >> 3)) * 8 + (is & 7);
            atomicOr(r.exc + (bit >> 5), 1u << (bit & 31));
        }
        const int cls = usex[ia] != 0 ? 0 : 1;
        r.X0[ray] = X0;
        r.S[ray] = S;
        r.code[ray] = (k0 <= k1 ? (k0 | (k1 << 15)) : kFpxEmpty) | (cls << 30) |
                      static_cast<int>(own ? kFpxExc : 0u);
        r.tie[ray] = tie;
    }
}

// Bounded wait until *p >= target (acquire, GPU scope); false after the
// wait limit.
__device__ __forceinline__ bool wait_count(const unsigned long long* p, unsigned long long target)
{
    auto ld = [&]() {
        unsigned long long v;
        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
        return v;
    };
    if (ld() >= target) return true;
    const unsigned long long t0 = global_ns();
    while (ld() < target) {
        if (global_ns() - t0 > kWaitLimitNs) return false;
        __nanosleep(100);
    }
    return true;
}

// Barrier 1 over the projector's consumer warps only (the producer warp runs on).
__device__ __forceinline__ void consumer_sync()
{
    asm volatile("bar.sync 1, %0;" ::"n"(kFpxWarps * 32) : "memory");
}

// The code of ray (ia, is): its own (flagged kFpxExc) where the exception
// bitmap says so, else the range of its view's model line.
__device__ __forceinline__ int ray_code(const FpxRays& r, const FpxConst& c, int ia, int is)
{
    const long long bit = (static_cast<long long>(ia) * c.octets + (is >> 3)) * 8 + (is & 7);
    const unsigned w = r.exc[bit >> 5];
    const FpxLine l = r.line[ia];
    if ((w >> (bit & 31)) & 1u) return r.code[static_cast<size_t>(ia) * c.ns + is];
    int k0, k1;
    view_range(l, is, c.n, &k0, &k1);
    return k0 | (k1 << 15);
}

template <int CH>
__global__ void __launch_bounds__(kFpxThreads, 1)
    fp_proj_f32(const float* __restrict__ img, float* __restrict__ imgT,
                float* __restrict__ proj, const FpxConst c, const FpxRays r,
                unsigned long long* __restrict__ tsync, unsigned long long ttarget)
{
    static_assert(CH >= 2 && CH % 2 == 0, "a chunk's rows are taken in pairs");
    extern __shared__ __align__(128) unsigned char fpx_dyn[];
    float* stage = reinterpret_cast<float*>(fpx_dyn + ((128u - (smem_u32(fpx_dyn) & 127u)) & 127u));
    __shared__ __align__(8) unsigned long long s_full[kFpxStages], s_empty[kFpxStages];
    __shared__ int s_work[kFpxRound];
    __shared__ int s_code[kFpxRound][32];           // ray codes of the round's slots
    __shared__ int s_assign[kFpxWarps][kFpxSlots];  // slot of the round, or -1
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = c.n;
    const long long item0 = static_cast<long long>(blockIdx.y) * n * n;
    const float* I = img + item0;
    // this CTA's slots: ci, ci + G, ci + 2G, ... of its class (count of them)
    const int G0 = r.cuts[0];
    const bool cls1 = static_cast<int>(blockIdx.x) >= G0;
    const int G = cls1 ? c.ctas - G0 : G0, ci = static_cast<int>(blockIdx.x) - (cls1 ? G0 : 0);
    const int s0 = (cls1 ? r.cuts[1] : 0) + ci, ncls = cls1 ? r.cuts[2] : r.cuts[1];
    const int count = ci < ncls ? (ncls - 1 - ci) / G + 1 : 0;
    const float* src = cls1 ? imgT : img;  // the staged array: rows are the marched lines
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < kFpxStages; ++s) {
            mbar_init(smem_u32(&s_full[s]), 1);
            mbar_init(smem_u32(&s_empty[s]), kFpxWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    // zero the stages once: the few slack elements past a band read as finite
    // (later bands leave image values there)
    for (int i = tid; i < kFpxStages * c.stage_floats; i += kFpxThreads) stage[i] = 0.0f;
    __syncthreads();

    if (tsync != nullptr && warp < kFpxWarps) {
        // Fused transposed copy (one image, cooperative launch): this CTA's
        // 32 x 32 tiles (blockIdx.x, + gridDim.x, ...) through shared memory,
        // then one count on tsync.  Column-marching CTAs stream imgT once the
        // count reaches ttarget (every CTA's tiles written).
        float(*t)[33] = reinterpret_cast<float(*)[33]>(&s_code[0][0]);
        const int tiles = (n + 31) / 32;
        for (int tb = blockIdx.x; tb < tiles * tiles; tb += gridDim.x) {
            const int x0 = (tb % tiles) * 32, y0 = (tb / tiles) * 32;
            for (int rr = warp; rr < 32; rr += kFpxWarps) {
                const int y = y0 + rr, x = x0 + lane;
                if (x < n && y < n) t[rr][lane] = img[static_cast<size_t>(y) * n + x];
            }
            consumer_sync();
            for (int rr = warp; rr < 32; rr += kFpxWarps) {
                const int x = x0 + rr, y = y0 + lane;
                if (x < n && y < n) imgT[static_cast<size_t>(x) * n + y] = t[lane][rr];
            }
            consumer_sync();
        }
        if (tid == 0) {
            // the copy's generic writes, released to the readers' bulk copies
            asm volatile("fence.proxy.async.global;" ::: "memory");
            __threadfence();
            atomicAdd(tsync, 1ull);
        }
    }

    int g = 0;  // band instances so far (producer and consumers count alike)
    for (int base = 0; base < count; base += kFpxRound) {
        const int m = min(kFpxRound, count - base);
        if (warp < kFpxWarps) {
            // the consumers prepare the round while the producer fills the stages
            for (int i = tid; i < kFpxRound; i += kFpxWarps * 32) (&s_assign[0][0])[i] = -1;
            // ---- ray codes and sample counts of the round's slots (slot warp + i *
            // kFpxWarps; the steps run over all of a warp's slots at once, so
            // their global loads overlap)
            int ia_[kFpxSlots], is_[kFpxSlots], code_[kFpxSlots];
#pragma unroll
            for (int i = 0; i < kFpxSlots; ++i) {
                const int t = warp + i * kFpxWarps;
                ia_[i] = -1;
                is_[i] = 0;
                if (t < m) slot_ray(static_cast<unsigned>(s0 + (base + t) * G), lane, c, r.views, &ia_[i], &is_[i]);
            }
#pragma unroll
            for (int i = 0; i < kFpxSlots; ++i)
                code_[i] = ia_[i] >= 0 && is_[i] < c.ns ? ray_code(r, c, ia_[i], is_[i]) : kFpxEmpty;
#pragma unroll
            for (int i = 0; i < kFpxSlots; ++i) {
                const int t = warp + i * kFpxWarps;
                if (t >= m) continue;
                s_code[t][lane] = code_[i];
                const int cnt = max(0, ((code_[i] >> 15) & 0x7FFF) - (code_[i] & 0x7FFF) + 1);
                const unsigned tot = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(cnt));
                if (lane == 0) s_work[t] = static_cast<int>(tot);
            }
            consumer_sync();
            // ---- deal the slots, largest first, to the warps in snake order
            if (tid < m) {
                const int wt = s_work[tid];
                int rk = 0;
                for (int u = 0; u < m; ++u) {
                    const int wu = s_work[u];
                    rk += (wu > wt || (wu == wt && u < tid)) ? 1 : 0;
                }
                const int k = rk / kFpxWarps, pos = rk - k * kFpxWarps;
                s_assign[(k & 1) ? kFpxWarps - 1 - pos : pos][k] = tid;
            }
            consumer_sync();
        }

        if (warp == kFpxWarps) {
            // ---- producer: one lane issues every band
            if (lane == 0) {
                bool alive = true;
                if (tsync != nullptr && cls1 && base == 0) {
                    // the fused transposed copy must be complete
                    if (!wait_count(tsync, ttarget)) {
                        raise_flag(kFlagWaitTimeout);
                        alive = false;
                    }
                    asm volatile("fence.proxy.async.global;" ::: "memory");
                }
                int g1 = g;
                for (int t = 0; alive && t < c.nbands; ++t, ++g1) {
                    const int s = g1 % kFpxStages;
                    const int use = g1 / kFpxStages;
                    if (use > 0 && !mbar_wait_bounded(smem_u32(&s_empty[s]), (use - 1) & 1)) {
                        raise_flag(kFlagWaitTimeout);
                        alive = false;
                        break;
                    }
                    const int nb = min(c.band, n - t * c.band);
                    const long long g0 = item0 + static_cast<long long>(t) * c.band * n;
                    const long long ga = g0 & ~3ll, gend = g0 + static_cast<long long>(nb) * n;
                    const long long gz = min((gend + 3) & ~3ll, c.total4);
                    const unsigned bytes = gz > ga ? static_cast<unsigned>((gz - ga) * sizeof(float)) : 0u;
                    float* dst = stage + s * c.stage_floats;
                    // the ragged tail of the array (not a 16-byte multiple) comes directly
                    for (long long i = max(c.total4, ga); i < min(gend, c.total); ++i) dst[i - ga] = src[i];
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_expect_tx(smem_u32(&s_full[s]), bytes);
                    if (bytes) bulk_load(smem_u32(dst), src + ga, bytes, smem_u32(&s_full[s]));
                }
                if (!alive) {
                    s_abort = 1;
                    // let the copies in flight land before the CTA moves on or exits
                    for (int gg = max(g, g1 - kFpxStages); gg < g1; ++gg)
                        mbar_wait_bounded(smem_u32(&s_full[gg % kFpxStages]), (gg / kFpxStages) & 1);
                }
            }
        } else {
            // ---- consumers: the assigned slots' rays in registers
            long long X0[kFpxSlots], S[kFpxSlots];
            int code[kFpxSlots];
            float sum[kFpxSlots];
#pragma unroll
            for (int j = 0; j < kFpxSlots; ++j) {
                X0[j] = 0;
                S[j] = 0;
                code[j] = kFpxEmpty;
                sum[j] = 0.0f;
                const int t = s_assign[warp][j];
                if (t >= 0) {
                    int ia, is;
                    slot_ray(static_cast<unsigned>(s0 + (base + t) * G), lane, c, r.views, &ia, &is);
                    if (ia >= 0 && is < c.ns) {
                        const int ray = ia * c.ns + is;
                        code[j] = s_code[t][lane];
                        if (static_cast<unsigned>(code[j]) & kFpxExc) {
                            X0[j] = r.X0[ray];
                            S[j] = r.S[ray];
                        } else {  // the view's model line
                            const FpxLine& l = r.line[ia];
                            X0[j] = l.x0 + static_cast<long long>(is) * l.d2;
                            S[j] = l.S;
                        }
                    }
                }
            }
            int g1 = g;
            bool alive = true;
            // constants of one_plus_frac held in registers: a value that came
            // through a shuffle is not re-read from the constant bank per use
            const unsigned fm = __shfl_sync(0xffffffffu, c.frac_mul, 0);
            const unsigned f1 = __shfl_sync(0xffffffffu, c.frac_one, 0);
            const float2 mone2 = make_float2(-1.0f, -1.0f);
            for (int t = 0; t < c.nbands; ++t, ++g1) {
                const int s = g1 % kFpxStages;
                int ok = 1;
                if (lane == 0) ok = mbar_wait_bounded(smem_u32(&s_full[s]), (g1 / kFpxStages) & 1);
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) {
                        raise_flag(kFlagWaitTimeout);
                        s_abort = 1;
                    }
                    alive = false;
                    break;
                }
                const int b0 = t * c.band, b1 = min(b0 + c.band, n) - 1;
                const long long g0 = item0 + static_cast<long long>(b0) * n;
                const float* bb = stage + s * c.stage_floats + (g0 & 3ll);
#pragma unroll
                for (int j = 0; j < kFpxSlots; ++j) {
                    // the lane's ray range [k0, k1] (empty: k0 above every row)
                    const int cj = code[j];
                    const int k0 = cj & 0x7FFF, k1 = (cj >> 15) & 0x7FFF;
                    if (!__any_sync(0xffffffffu, k0 <= b1 && k1 >= b0)) continue;
                    // sample b0 at row 0 of the band; a row step adds n to the word
                    // offset, so the integer part is the staged index
                    long long x = X0[j] + static_cast<long long>(b0) * S[j];
                    const long long S2 = S[j] + (static_cast<long long>(n) << 32);
                    float a = 0.0f, b = 0.0f;  // this band's partial sums (blocked summation)
                    for (int r0 = b0; r0 <= b1; r0 += CH) {
                        if (__all_sync(0xffffffffu, k0 <= r0 && k1 >= r0 + CH - 1)) {
                            // every lane's ray covers the chunk: no per-sample test.
                            // Even and odd rows run as two independent chains
                            // (positions and sums) whose FP32 work is packed in
                            // pairs (even row in .x), unrolled by 4 row pairs only:
                            // every slot's fully unrolled chunk would outgrow the
                            // instruction cache.
                            long long xo = x + S2;
                            const long long S4 = S2 + S2;
                            float2 a2 = make_float2(0.0f, 0.0f), b2 = a2;
#pragma unroll 4
                            for (int r = 0; r < CH; r += 2) {
                                const float* pe = bb + static_cast<int>(x >> 32);
                                const float* po = bb + static_cast<int>(xo >> 32);
                                const float2 p0 = make_float2(pe[0], po[0]);
                                const float2 p1 = make_float2(pe[1], po[1]);
                                const float2 u = __fadd2_rn(
                                    make_float2(one_plus_frac(x, fm, f1), one_plus_frac(xo, fm, f1)), mone2);
                                a2 = __fadd2_rn(a2, p0);
                                b2 = __ffma2_rn(u, f2_sub(p1, p0), b2);
                                x += S4;
                                xo += S4;
                            }
                            a += a2.x + a2.y;
                            b += b2.x + b2.y;
                        } else {
                            // the lane's own rows of the chunk (a divergent loop)
                            const int ka = max(k0, r0), kb = min(k1, r0 + CH - 1);
                            long long y = x + static_cast<long long>(ka - r0) * S2;
#pragma unroll 1
                            for (int k = ka; k <= kb; ++k) {
                                const float* p = bb + static_cast<int>(y >> 32);
                                const float p0 = p[0], p1 = p[1];
                                a += p0;
                                b = fmaf(one_plus_frac(y, fm, f1) - 1.0f, p1 - p0, b);
                                y += S2;
                            }
                            x += static_cast<long long>(CH) * S2;
                        }
                    }
                    sum[j] += a + b;
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(smem_u32(&s_empty[s]));
            }
            // ---- results (every ray of an assigned slot, also one with no valid sample)
#pragma unroll
            for (int j = 0; j < kFpxSlots; ++j) {
                const int t = s_assign[warp][j];
                if (!alive || t < 0) continue;
                int ia, is;
                slot_ray(static_cast<unsigned>(s0 + (base + t) * G), lane, c, r.views, &ia, &is);
                if (ia < 0 || is >= c.ns) continue;
                float v = sum[j];
                const int gi = (static_cast<unsigned>(code[j]) & kFpxExc) ? r.tie[ia * c.ns + is] : -1;
                if (gi >= 0) {
                    // border samples of a tie ray found inside by the reference's
                    // rule: read directly
                    const FpxTie& tt = r.ties[gi];
                    for (int a = 0; a < tt.namb; ++a) {
                        if (!((tt.in >> a) & 1u)) continue;
                        const int k = tt.amb[a];
                        const long long X = X0[j] + static_cast<long long>(k) * S[j];
                        int hi = static_cast<int>(X >> 32);
                        float u = frac_of(X);
                        if (X < 0) {
                            hi = 0;
                            u = 0.0f;
                        } else if (hi >= n - 1) {
                            hi = n - 1;
                            u = 0.0f;
                        }
                        // row ray: row k, columns hi, hi + 1; column ray: column k, rows hi, hi + 1
                        const size_t i0 = cls1 ? static_cast<size_t>(hi) * n + k : static_cast<size_t>(k) * n + hi;
                        const size_t d1 = cls1 ? static_cast<size_t>(n) : 1;
                        const float p0 = I[i0], p1 = u > 0.0f ? I[i0 + d1] : p0;
                        v += p0 + u * (p1 - p0);
                    }
                }
                proj[blockIdx.y * c.proj_stride + static_cast<size_t>(ia) * c.ns + is] = v * r.vw[ia];
            }
        }
        g += c.nbands;
        __syncthreads();  // round end: every copy consumed; the next round may rewrite the tables
        if (s_abort) break;
    }
}

// ---- FP32 adjoint: per-pixel gather over each view's channel footprint ----
// Channel positions of pixel centres are 32.32 fixed point built from the
// caller's grad-prep table (one conversion per tile line and view); the
// footprint and triangle weights are those of src/fp_par_2d.cc:339-383:
// channels within |offset| of the pixel's position mid, weight 1 - |mid - is| /
// |offset|.
//
// Interior pixels of views with |offset| <= 1 (every view when dx, dy <= ds)
// touch at most channels floor(mid) and floor(mid) + 1, whose weights follow
// from the fraction with two FMAs (saturated: both are at most 1, and the
// clamp at 0 is the footprint's edge).  Once per call, fp_adj_prep converts
// the caller's positions to 32.32 fixed point and fp_adj_windows finds, per
// (view, tile), the channel window the tile's pixels fall in.  fp_adj_f32
// stages, per block of views, each window as zero-padded pairs (w p[i],
// w p[i+1]) of IMG images side by side (w = the view weight), so a pixel-view
// of IMG images is one shared load, a fraction and two weights shared by the
// images, and two FMAs per image; positions advance by 64-bit adds.  It
// computes every pixel that way.  Pixels on the image border have one-sided
// footprints (channels on the neighbour's side only); fp_adj_border_f32 then
// recomputes those 4n - 4 pixels exactly and overwrites them.  When one image's
// tiles would not fill the GPU, each tile's views are split into segments whose
// partial images fp_adj_reduce sums in segment order.
// Views with |offset| > 1 or a window wider than the staged one take the exact
// per-pixel path in both kernels.
constexpr int kFaViews = 16;
constexpr int kFaTileX = 32;
// Tile of ROWS pixels of one column per thread: 32 x 8*ROWS pixels, 256 threads.
template <int ROWS>
struct FaShape {
    static constexpr int TY = 8 * ROWS;
    static constexpr int LINES = TY > kFaTileX ? TY : kFaTileX;  // rows or columns of a tile
    static constexpr int WIN = 2 * LINES;                        // staged channel pairs per view
};
// Units of 2^-32 channel within which a border pixel's position counts as on a
// channel: the fixed-point position is within 0.5 + 0.5*along units of the
// reference's FP64 one (along < 8192).
constexpr unsigned kFaTie = 8192;

// 32.32 fixed point of a table value: integer conversion where exact, FP64 beyond.
__device__ __forceinline__ long long fix32_any(double v)
{
    return ((double_bits(v) >> 52) & 0x7FF) < 1043 ? fix32(v) : llrint(v * kTwo32);
}

// The reference grad's taps for one pixel-view: MID = the pixel's position
// (fixed point), O1 = the view's offset, `along` = the pixel's index along its
// line, pp = the caller's (begin, offset) of the pixel's line.  A border pixel's
// footprint is one-sided (toward the neighbour pixel); its end channel is
// decided from the fixed-point fraction or, when mid lies within kFaTie units
// of a channel, in FP64 exactly as the reference does.  Either two taps at mi,
// mi + 1 with weights w0, w1, or channels lo..hi with weight 1 - |mid - is| / |o|.
struct AdjTap {
    int mi, lo, hi;
    float mf, w0, w1;
    bool two;
};

__device__ __forceinline__ AdjTap adj_tap_plan(long long MID, long long O1, float inv, bool two, int along,
                                               int n, int ns, const double* __restrict__ pp)
{
    AdjTap t;
    t.mi = static_cast<int>(MID >> 32);
    t.mf = frac_of(MID);
    const bool border = along == 0 || along == n - 1;
    const unsigned frac_bits = static_cast<unsigned>(MID);
    const bool tie = border && (n == 1 || frac_bits < kFaTie || frac_bits > 0u - kFaTie);
    t.two = two && !tie;
    if (t.two) {
        t.w0 = fmaxf(fmaf(-t.mf, inv, 1.0f), 0.0f);
        t.w1 = fmaxf(fmaf(t.mf, inv, 1.0f - inv), 0.0f);
        if (border) {
            const bool ge = (along == 0) != (O1 < 0);  // footprint [mid, mid + |o|]
            if (ge) t.w0 = 0.0f;
            else t.w1 = 0.0f;
        }
        t.lo = t.hi = 0;
        return t;
    }
    t.w0 = t.w1 = 0.0f;
    long long L = along == 0 ? MID : MID - O1;
    long long R = along == n - 1 ? MID : MID + O1;
    if (L > R) {
        const long long x = L;
        L = R;
        R = x;
    }
    t.lo = max(static_cast<int>((L + 0xFFFFFFFFll) >> 32), 0);
    t.hi = min(static_cast<int>(R >> 32), ns - 1);
    if (border) {
        // the end channel sits at the pixel itself with weight ~1: the range
        // is decided in FP64 as the reference does (mid = begin + offset*along)
        const double off = pp[1];
        const double mid = __dadd_rn(pp[0], __dmul_rn(off, static_cast<double>(along)));
        double left = along == 0 ? mid : __dsub_rn(mid, off);
        double right = along == n - 1 ? mid : __dadd_rn(mid, off);
        if (left > right) {
            const double x = left;
            left = right;
            right = x;
        }
        t.lo = static_cast<int>(fmax(ceil(left), 0.0));
        t.hi = static_cast<int>(fmin(floor(right), static_cast<double>(ns - 1)));
    }
    return t;
}

// The tap sum of one detector row.
__device__ __forceinline__ float adj_tap_apply(const float* __restrict__ row, const AdjTap& t, float inv, int ns)
{
    if (t.two) {
        const float p0 = static_cast<unsigned>(t.mi) < static_cast<unsigned>(ns) ? __ldg(row + t.mi) : 0.0f;
        const float p1 = static_cast<unsigned>(t.mi + 1) < static_cast<unsigned>(ns) ? __ldg(row + t.mi + 1) : 0.0f;
        return fmaf(t.w0, p0, t.w1 * p1);
    }
    float part = 0.0f;
    for (int is = t.lo; is <= t.hi; ++is) {
        const float d = fabsf(t.mf - static_cast<float>(is - t.mi));
        part = fmaf(fmaf(-d, inv, 1.0f), __ldg(row + is), part);
    }
    return part;
}

// Per-view constants of the adjoint, from the caller's grad-prep tables.
struct AdjView {
    long long O1;  // offset, 32.32 fixed point
    float inv;     // 1 / |offset|
    float w;       // view weight
    int ux;        // lines are rows
    int two;       // |offset| <= 1
};

// Channel window of one (view, tile): pairs lo .. lo + width - 1 are staged;
// width 0 = the view takes the exact path on this tile.
struct AdjWin {
    int lo;
    int width;
};

// One pass over the grad-prep tables per call: the 32.32 fixed-point begin of
// every (view, line) and the per-view constants, so the gather's CTAs (and
// batch items) load them instead of converting the FP64 values themselves.
__global__ void __launch_bounds__(256)
    fp_adj_prep(const double* __restrict__ weights, const double* __restrict__ pos,
                const int* __restrict__ usex, long long* __restrict__ B, AdjView* __restrict__ V,
                int na, int n)
{
    const long long i = static_cast<long long>(blockIdx.x) * 256 + threadIdx.x;
    if (i >= static_cast<long long>(na) * n) return;
    const double* pp = pos + i * 2;
    B[i] = fix32_any(pp[0]);
    if (i % n == 0) {
        const int ia = static_cast<int>(i / n);
        const float o1 = fabsf(dbl2flt(pp[1]));
        AdjView v;
        v.O1 = fix32_any(pp[1]);
        v.inv = 1.0f / o1;
        v.w = dbl2flt(weights[ia]);
        v.ux = usex[ia] != 0;
        v.two = o1 <= 1.0f;
        V[ia] = v;
    }
}

// The channel window of every (view, tile).  For a fixed line the position is
// linear in `along`, so over a tile it spans [B_l + min(a0, a1), B_l + max(a0,
// a1)], a0 and a1 the offsets of the tile's first and last along index; over
// the tile's lines that is [Bmin + min(a0, a1), Bmax + max(a0, a1)], Bmin and
// Bmax the extremes of the line positions of the tile's band (a row band of
// row-marching views, else a column band; lines past the image repeat the last
// one, as the gather's line positions do).  One warp per (view, band): the
// band's extremes, then the window of each tile of the band.  Windows are
// shared by every image of the batch.
__global__ void __launch_bounds__(256)
    fp_adj_windows(const long long* __restrict__ B, const AdjView* __restrict__ V,
                   AdjWin* __restrict__ W, int na, int n, int tiles_x, int tiles_y, int ty, int win)
{
    const int nbmax = max(tiles_x, tiles_y);
    const long long wid = (static_cast<long long>(blockIdx.x) * 256 + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= static_cast<long long>(na) * nbmax) return;  // warp-uniform
    const int ia = static_cast<int>(wid / nbmax), band = static_cast<int>(wid - static_cast<long long>(ia) * nbmax);
    const AdjView v = V[ia];
    if (band >= (v.ux ? tiles_y : tiles_x)) return;  // warp-uniform
    const int lines = v.ux ? ty : kFaTileX;
    long long bmin = LLONG_MAX, bmax = LLONG_MIN;
    for (int l = lane; l < lines; l += 32) {
        const long long b = __ldg(B + static_cast<size_t>(ia) * n + min(band * lines + l, n - 1));
        bmin = b < bmin ? b : bmin;
        bmax = b > bmax ? b : bmax;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long x = __shfl_xor_sync(0xffffffffu, bmin, o);
        const long long y = __shfl_xor_sync(0xffffffffu, bmax, o);
        bmin = x < bmin ? x : bmin;
        bmax = y > bmax ? y : bmax;
    }
    const int ntiles = tiles_x * tiles_y;
    const int alen = v.ux ? kFaTileX : ty;
    const int count = v.ux ? tiles_x : tiles_y;
    for (int k = lane; k < count; k += 32) {
        const long long a0 = static_cast<long long>(k * alen) * v.O1;
        const long long a1 = a0 + static_cast<long long>(alen - 1) * v.O1;
        const int lo = static_cast<int>((bmin + (a0 < a1 ? a0 : a1)) >> 32);
        const int hi = static_cast<int>((bmax + (a0 < a1 ? a1 : a0)) >> 32);
        const int t = v.ux ? band * tiles_x + k : k * tiles_x + band;
        const long long width = static_cast<long long>(hi) - lo + 1;
        W[static_cast<size_t>(ia) * ntiles + t] = AdjWin{lo, v.two && width <= win ? static_cast<int>(width) : 0};
    }
}

// One staged pixel-view of IMG images: pair entry at `a` holds (w p[m], w p[m+1])
// of each image, m = floor(MID).
template <int IMG, int ROWS>
__device__ __forceinline__ void adj_tap_staged(float (&blk)[IMG][ROWS], int r, long long MID, unsigned pb,
                                               float inv, float inv1)
{
    const float mf = frac_of(MID);
    const float w0 = __saturatef(fmaf(-mf, inv, 1.0f));
    const float w1 = __saturatef(fmaf(mf, inv, inv1));
    const unsigned a = pb + 8u * IMG * static_cast<unsigned>(MID >> 32);
    if constexpr (IMG == 1) {
        float2 p;
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(p.x), "=f"(p.y) : "r"(a));
        blk[0][r] = fmaf(w0, p.x, fmaf(w1, p.y, blk[0][r]));
    } else {
#pragma unroll
        for (int h = 0; h < IMG / 2; ++h) {
            float4 p;
            asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                         : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w)
                         : "r"(a + 16u * h));
            blk[2 * h][r] = fmaf(w0, p.x, fmaf(w1, p.y, blk[2 * h][r]));
            blk[2 * h + 1][r] = fmaf(w0, p.z, fmaf(w1, p.w, blk[2 * h + 1][r]));
        }
    }
}

// The gather: CTA = one 32 x 8*ROWS tile of IMG images and one segment of
// seg_len views: blockIdx.z = group * segs + segment, images img0 + group*IMG ...
// With one segment it writes the images; with several, segment s writes its
// partial sums to part[s][image] for fp_adj_reduce.  Per block of kFaViews views: one phase loads the tile's line positions and
// the windows' pairs (all loads in flight), one barrier, compute, one barrier;
// the next block's view constants and windows are copied (cp.async) during
// the compute into the other half of s_v / s_w.
template <int ROWS, int IMG>
__global__ void __launch_bounds__(256, ROWS * IMG >= 32 ? 2 : 3)
    fp_adj_f32(const float* __restrict__ proj, float* __restrict__ img, const long long* __restrict__ B,
               const AdjView* __restrict__ V, const AdjWin* __restrict__ W, const double* __restrict__ pos,
               const FpConst c, int img0, int segs, int seg_len, float* __restrict__ part, int batch)
{
    using S = FaShape<ROWS>;
    constexpr int TY = S::TY, LINES = S::LINES, WIN = S::WIN;
    static_assert(IMG == 1 || IMG == 2 || IMG == 4, "images per CTA");
    __shared__ long long s_base[kFaViews][LINES];
    __shared__ AdjView s_v[2][kFaViews];
    __shared__ AdjWin s_w[2][kFaViews];
    extern __shared__ __align__(16) float s_pair_dyn[];  // [kFaViews][WIN][2 * IMG]
    float(*s_pair)[WIN][2 * IMG] = reinterpret_cast<float(*)[WIN][2 * IMG]>(s_pair_dyn);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tx0 = blockIdx.x * kFaTileX, ty0 = blockIdx.y * TY;
    const int ix = tx0 + lane;
    const int ntiles = gridDim.x * gridDim.y, tile = blockIdx.y * gridDim.x + blockIdx.x;
    const int seg = blockIdx.z % segs, im = img0 + (blockIdx.z / segs) * IMG;
    const int vb = seg * seg_len, ve = min(c.na, vb + seg_len);
    const float* P = proj + static_cast<size_t>(im) * c.proj_stride;
    const int n = c.nx;  // == ny
    const int ns = c.ns;
    float acc[IMG][ROWS];
#pragma unroll
    for (int i = 0; i < IMG; ++i)
#pragma unroll
        for (int r = 0; r < ROWS; ++r) acc[i][r] = 0.0f;

    if (tid < min(kFaViews, ve - vb)) {
        s_v[0][tid] = V[vb + tid];
        s_w[0][tid] = W[static_cast<size_t>(vb + tid) * ntiles + tile];
    }
    __syncthreads();
    int buf = 0;
    for (int v0 = vb; v0 < ve; v0 += kFaViews, buf ^= 1) {
        const int nv = min(kFaViews, ve - v0);
        // the next block's view constants and windows, copied during this
        // block into the other half of s_v / s_w (last read before this
        // block's first barrier)
        const int vn = v0 + kFaViews + tid;
        if (tid < kFaViews && vn < ve) {
            static_assert(sizeof(AdjView) == 24 && sizeof(AdjWin) == 8, "8-byte copies");
            const unsigned dv = smem_u32(&s_v[buf ^ 1][tid]);
            const char* sv = reinterpret_cast<const char*>(V + vn);
            cp_async8(dv, sv);
            cp_async8(dv + 8, sv + 8);
            cp_async8(dv + 16, sv + 16);
            cp_async8(smem_u32(&s_w[buf ^ 1][tid]), W + static_cast<size_t>(vn) * ntiles + tile);
        }
        // line positions of the tile: rows for row-marching views, else columns
#pragma unroll
        for (int it = 0; it < kFaViews * LINES / 256; ++it) {
            const int idx = it * 256 + tid;
            const int j = idx / LINES, l = idx - j * LINES;
            if (j < nv) {
                const int ux = s_v[buf][j].ux;
                if (l < (ux ? TY : kFaTileX))
                    s_base[j][l] = __ldg(B + static_cast<size_t>(v0 + j) * n + min((ux ? ty0 : tx0) + l, n - 1));
            }
        }
        // staged windows: (w p[lo+k], w p[lo+k+1]) per image, zero off the detector
#pragma unroll
        for (int it = 0; it < kFaViews * WIN / 256; ++it) {
            const int idx = it * 256 + tid;
            const int j = idx / WIN, k = idx - j * WIN;
            if (j < nv && k < s_w[buf][j].width) {
                const float w = s_v[buf][j].w;
                const int g = s_w[buf][j].lo + k;
                const bool in0 = static_cast<unsigned>(g) < static_cast<unsigned>(ns);
                const bool in1 = static_cast<unsigned>(g + 1) < static_cast<unsigned>(ns);
                const float* row = P + static_cast<size_t>(v0 + j) * ns;
                float e[2 * IMG];
#pragma unroll
                for (int i = 0; i < IMG; ++i) {
                    e[2 * i] = in0 ? __ldg(row + i * c.proj_stride + g) * w : 0.0f;
                    e[2 * i + 1] = in1 ? __ldg(row + i * c.proj_stride + g + 1) * w : 0.0f;
                }
                if constexpr (IMG == 1) {
                    *reinterpret_cast<float2*>(&s_pair[j][k][0]) = make_float2(e[0], e[1]);
                } else {
#pragma unroll
                    for (int h = 0; h < IMG / 2; ++h)
                        *reinterpret_cast<float4*>(&s_pair[j][k][4 * h]) =
                            make_float4(e[4 * h], e[4 * h + 1], e[4 * h + 2], e[4 * h + 3]);
                }
            }
        }
        __syncthreads();
        float blk[IMG][ROWS];  // this view block's partial sums (blocked summation)
#pragma unroll
        for (int i = 0; i < IMG; ++i)
#pragma unroll
            for (int r = 0; r < ROWS; ++r) blk[i][r] = 0.0f;
        for (int j = 0; j < nv; ++j) {
            const AdjView v = s_v[buf][j];
            const AdjWin wn = s_w[buf][j];
            if (wn.width > 0) {
                const float inv1 = 1.0f - v.inv;
                const unsigned pb = smem_u32(&s_pair[j][0][0]) - 8u * IMG * static_cast<unsigned>(wn.lo);
                if (v.ux) {  // along = ix, line = row
                    const long long A = static_cast<long long>(ix) * v.O1;
#pragma unroll
                    for (int r = 0; r < ROWS; ++r)
                        adj_tap_staged<IMG, ROWS>(blk, r, s_base[j][warp * ROWS + r] + A, pb, v.inv, inv1);
                } else {     // along = row, line = ix
                    long long MID = s_base[j][lane] + static_cast<long long>(ty0 + warp * ROWS) * v.O1;
#pragma unroll
                    for (int r = 0; r < ROWS; ++r) {
                        adj_tap_staged<IMG, ROWS>(blk, r, MID, pb, v.inv, inv1);
                        MID += v.O1;
                    }
                }
            } else {
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int iy = ty0 + warp * ROWS + r;
                    const int along = v.ux ? ix : iy;
                    const int lin = v.ux ? iy : ix;
                    const long long MID = s_base[j][v.ux ? warp * ROWS + r : lane] +
                                          static_cast<long long>(along) * v.O1;
                    const double* pp = pos + (static_cast<size_t>(v0 + j) * n + min(lin, n - 1)) * 2;
                    const AdjTap t = adj_tap_plan(MID, v.O1, v.inv, v.two != 0, along, n, ns, pp);
#pragma unroll
                    for (int i = 0; i < IMG; ++i) {
                        const float* row = P + i * c.proj_stride + static_cast<size_t>(v0 + j) * ns;
                        blk[i][r] = fmaf(adj_tap_apply(row, t, v.inv, ns), v.w, blk[i][r]);
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < IMG; ++i)
#pragma unroll
            for (int r = 0; r < ROWS; ++r) acc[i][r] += blk[i][r];
        cp_async_wait_all();
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < IMG; ++i) {
        float* O = segs == 1 ? img + static_cast<size_t>(im + i) * c.img_stride
                             : part + (static_cast<size_t>(seg) * batch + im + i) * c.img_stride;
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int iy = ty0 + warp * ROWS + r;
            if (ix < c.nx && iy < c.ny) O[static_cast<size_t>(iy) * c.nx + ix] = acc[i][r];
        }
    }
}

// Sum of the segments' partial images in segment order: img[e] = part[0][e] +
// part[1][e] + ..., `count` = floats of the batch, as float4 when `vec`.
__global__ void __launch_bounds__(256)
    fp_adj_reduce(const float* __restrict__ part, float* __restrict__ img, size_t count, int segs, bool vec)
{
    const size_t stride = static_cast<size_t>(gridDim.x) * 256;
    if (vec) {
        const float4* P4 = reinterpret_cast<const float4*>(part);
        float4* O4 = reinterpret_cast<float4*>(img);
        const size_t n4 = count / 4;
        for (size_t e = blockIdx.x * 256ull + threadIdx.x; e < n4; e += stride) {
            float4 a = P4[e];
            for (int s = 1; s < segs; ++s) {
                const float4 b = P4[s * n4 + e];
                a.x += b.x;
                a.y += b.y;
                a.z += b.z;
                a.w += b.w;
            }
            O4[e] = a;
        }
    } else {
        for (size_t e = blockIdx.x * 256ull + threadIdx.x; e < count; e += stride) {
            float a = part[e];
            for (int s = 1; s < segs; ++s) a += part[s * count + e];
            img[e] = a;
        }
    }
}

// The 4n - 4 border pixels, exactly, overwriting fp_adj_f32's values: one
// 128-thread block per pixel and up to kFbImg images (blockIdx.y*kFbImg ..).
// Thread t sums views t, t+128, ... of each image (the taps of a view are
// planned once for all images), then a fixed tree: a shuffle tree per warp,
// the four warps in order.
constexpr int kFbImg = 8;
__global__ void __launch_bounds__(128)
    fp_adj_border_f32(const float* __restrict__ proj, float* __restrict__ img,
                      const long long* __restrict__ B, const AdjView* __restrict__ V,
                      const double* __restrict__ pos, const FpConst c, int batch)
{
    __shared__ float s_part[4][kFbImg];
    const int n = c.nx, ns = c.ns;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int b = blockIdx.x;
    int ix, iy;
    if (b < n) {
        ix = b;
        iy = 0;
    } else if (b < 2 * n) {
        ix = b - n;
        iy = n - 1;
    } else if (b < 3 * n - 2) {
        ix = 0;
        iy = b - 2 * n + 1;
    } else {
        ix = n - 1;
        iy = b - 3 * n + 3;
    }
    const int im0 = blockIdx.y * kFbImg;
    const int cnt = min(kFbImg, batch - im0);
    const float* P = proj + static_cast<size_t>(im0) * c.proj_stride;
    float acc[kFbImg];
#pragma unroll
    for (int i = 0; i < kFbImg; ++i) acc[i] = 0.0f;
    for (int ia = threadIdx.x; ia < c.na; ia += 128) {
        const AdjView v = V[ia];
        const int along = v.ux ? ix : iy, lin = v.ux ? iy : ix;
        const size_t line = static_cast<size_t>(ia) * n + lin;
        const long long MID = __ldg(B + line) + static_cast<long long>(along) * v.O1;
        const AdjTap t = adj_tap_plan(MID, v.O1, v.inv, v.two != 0, along, n, ns, pos + line * 2);
        const float* row = P + static_cast<size_t>(ia) * ns;
        if (t.two) {  // every image's two loads issued before the first FMA
            const bool in0 = static_cast<unsigned>(t.mi) < static_cast<unsigned>(ns);
            const bool in1 = static_cast<unsigned>(t.mi + 1) < static_cast<unsigned>(ns);
            float p0[kFbImg], p1[kFbImg];
#pragma unroll
            for (int i = 0; i < kFbImg; ++i) {
                const float* r = row + i * c.proj_stride;
                p0[i] = i < cnt && in0 ? __ldg(r + t.mi) : 0.0f;
                p1[i] = i < cnt && in1 ? __ldg(r + t.mi + 1) : 0.0f;
            }
#pragma unroll
            for (int i = 0; i < kFbImg; ++i) acc[i] = fmaf(fmaf(t.w0, p0[i], t.w1 * p1[i]), v.w, acc[i]);
        } else {
#pragma unroll
            for (int i = 0; i < kFbImg; ++i)
                if (i < cnt) acc[i] = fmaf(adj_tap_apply(row + i * c.proj_stride, t, v.inv, ns), v.w, acc[i]);
        }
    }
#pragma unroll
    for (int i = 0; i < kFbImg; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
        if (lane == 0) s_part[warp][i] = acc[i];
    }
    __syncthreads();
    if (threadIdx.x < cnt) {
        const int i = threadIdx.x;
        const float sum = ((s_part[0][i] + s_part[1][i]) + s_part[2][i]) + s_part[3][i];
        img[static_cast<size_t>(im0 + i) * c.img_stride + static_cast<size_t>(iy) * n + ix] = sum;
    }
}

constexpr int kFp64Threads = 128;

template <typename T>
__global__ void __launch_bounds__(kFp64Threads)
    fp_ray_kernel(const T* __restrict__ img, T* __restrict__ proj,
                  const double* __restrict__ sincos, const double* __restrict__ bo,
                  const int* __restrict__ usex, int ns, int na, int nx, int ny, double dx,
                  double dy, size_t img_stride, size_t proj_stride)
{
    const int is = blockIdx.x * kFp64Threads + threadIdx.x;
    const int ia = blockIdx.y;
    if (is >= ns) return;
    const T* I = img + blockIdx.z * img_stride;
    const size_t ray = static_cast<size_t>(ia) * ns + is;
    const bool ux = usex[ia] != 0;
    const double begin = bo[2 * ray], step = bo[2 * ray + 1];
    const int nsamp = ux ? ny : nx;
    const int lim = ux ? nx - 1 : ny - 1;
    T sum = 0;
    {
        double x = begin;
        for (int k = 0; k < nsamp; ++k) {
            if (x >= 0 && x <= lim) {
                const int i1 = static_cast<int>(floor(x));
                const int i2 = static_cast<int>(ceil(x));
                const double u = x - i1;
                if (ux)
                    sum += (1 - u) * I[i1 + static_cast<size_t>(k) * nx] + u * I[i2 + static_cast<size_t>(k) * nx];
                else
                    sum += (1 - u) * I[k + static_cast<size_t>(i1) * nx] + u * I[k + static_cast<size_t>(i2) * nx];
            }
            x += step;
        }
    }
    const double dw = ux ? fabs(dy / sincos[2 * ia + 1]) : fabs(dx / sincos[2 * ia]);
    proj[blockIdx.z * proj_stride + ray] = static_cast<T>(sum * static_cast<T>(dw));
}

template <typename T>
__global__ void fp_adj_kernel(const T* __restrict__ proj, T* __restrict__ img,
                              const double* __restrict__ weights, const double* __restrict__ pos,
                              const int* __restrict__ usex, int ns, int na, int nx, int ny,
                              size_t proj_stride, size_t img_stride)
{
    const int ix = blockIdx.x * 32 + threadIdx.x;
    const int iy = blockIdx.y * 8 + threadIdx.y;
    if (ix >= nx || iy >= ny) return;
    const T* P = proj + blockIdx.z * proj_stride;
    double sum = 0.0;
    for (int ia = 0; ia < na; ++ia) {
        const bool ux = usex[ia] != 0;
        const double* pp = pos + static_cast<size_t>(ia) * 2 * nx;
        const int lin = ux ? iy : ix;   // table entry
        const int along = ux ? ix : iy; // position along the entry
        const int last = ux ? nx - 1 : ny - 1;
        T begin, step;
        begin = static_cast<T>(pp[2 * lin]);
        step = static_cast<T>(pp[2 * lin + 1]);
        const T mid = begin + step * static_cast<T>(along);
        T left = along == 0 ? mid : mid - step;
        T right = along == last ? mid : mid + step;
        if (left > right) {
            const T t = left;
            left = right;
            right = t;
        }
        T lo = ceil(left), hi = floor(right);
        if (lo < 0) lo = 0;
        if (hi > static_cast<T>(ns - 1)) hi = static_cast<T>(ns - 1);
        const T* row = P + static_cast<size_t>(ia) * ns;
        const T inv = static_cast<T>(1) / step;
        T part = 0;
        for (int is = static_cast<int>(lo); is <= static_cast<int>(hi); ++is) {
            const T t = (mid - static_cast<T>(is)) * inv;
            part += (static_cast<T>(1) - (t < 0 ? -t : t)) * row[is];
        }
        sum += static_cast<double>(part) * weights[ia];
    }
    img[blockIdx.z * img_stride + static_cast<size_t>(iy) * nx + ix] = static_cast<T>(sum);
}

int check_fp(const ctr_par_param* p, const void* a, const void* b, const void* t0,
             const void* t1, const void* t2, int batch)
{
    if (!p || !a || !b || !t0 || !t1 || !t2) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->na < 1 || p->nx < 1 || p->ny < 1) return fail(CTR_ERR_INVALID_ARG, "empty geometry");
    if (p->nx != p->ny) return fail(CTR_ERR_INVALID_ARG, "ray-driven projection needs nx == ny");
    if (batch > 65535 || p->na > 65535) return fail(CTR_ERR_UNSUPPORTED, "batch or na > 65535");
    return CTR_OK;
}

FpConst fp_const(const ctr_par_param* p)
{
    FpConst c{};
    c.ns = p->ns; c.na = p->na; c.nx = p->nx; c.ny = p->ny;
    c.dx = p->dx; c.dy = p->dy;
    c.img_stride = static_cast<size_t>(p->nx) * p->ny;
    c.proj_stride = static_cast<size_t>(p->ns) * p->na;
    return c;
}

// FpxConst of the pipelined FP32 forward projector, or false when the geometry
// needs the plain band kernel (very wide images, a misaligned image, more
// slots than 32-bit slot indices hold).
bool fpx_const(const ctr_par_param* p, const void* img, int batch, FpxConst* out, size_t* smem)
{
    const int n = static_cast<int>(p->nx);
    if (n > 8192 || reinterpret_cast<uintptr_t>(img) % 16 != 0) return false;
    FpxConst c{};
    c.ns = p->ns;
    c.na = p->na;
    c.n = n;
    c.octets = static_cast<int>(div_up(p->ns, 8));
    c.stride = std::max(1, static_cast<int>(0.618 * c.octets + 0.5));
    while (std::gcd(c.stride, c.octets) != 1) ++c.stride;
    c.quads = static_cast<int>(div_up(p->na, 4));
    const long long slots = static_cast<long long>(c.quads + 2) * c.octets;  // with class padding
    if (slots >= (1ll << 30) || static_cast<long long>(p->na) * p->ns >= (1ll << 31)) return false;
    // one CTA an SM while every CTA's slots fit one round; else enough CTAs
    // for rounds 7/8 full
    int dev = 0;
    c.sms = kSmCount;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        c.sms = kSmCount;
    const long long ctas = div_up(slots, c.sms) <= kFpxRound ? static_cast<long long>(c.sms) : div_up(slots * 8, kFpxRound * 7);
    c.ctas = static_cast<int>(std::min<long long>(ctas, slots));
    // rows per stage: a multiple of the projector's chunk of 16, 8 or 2 rows
    // (the chunk's rows are taken in pairs, so never fewer than 2)
    c.band = std::max(1, std::min(32, kFpxStageFloats / n));
    c.band = c.band >= 16 ? c.band / 16 * 16 : (c.band >= 8 ? 8 : c.band & ~1);
    if (c.band < 2) return false;
    c.nbands = static_cast<int>(div_up(n, c.band));
    c.stage_floats = (c.band * n + 8 + 31) / 32 * 32;
    c.total = static_cast<long long>(batch) * n * n;
    c.total4 = c.total & ~3ll;
    c.proj_stride = static_cast<size_t>(p->ns) * p->na;
    c.dx = static_cast<float>(p->dx);
    c.dy = static_cast<float>(p->dy);
    c.frac_mul = 1u << 23;
    c.frac_one = 0x3F800000u;
    *smem = 128 + static_cast<size_t>(kFpxStages) * c.stage_floats * sizeof(float);
    if (*smem > 200 * 1024) return false;
    *out = c;
    return true;
}

// Bytes of scratch the projector needs: the transposed image, then its tables.
size_t fpx_scratch_bytes(const FpxConst& c)
{
    const size_t imgT = (static_cast<size_t>(c.total) * sizeof(float) + 255) & ~static_cast<size_t>(255);
    return imgT + fpx_table_bytes(static_cast<long long>(c.na) * c.ns, c.na, c.ctas);
}

// Carves the ray tables out of `b` (256-byte aligned).
FpxRays fpx_tables(unsigned char* b, const FpxConst& c)
{
    const size_t rays = static_cast<size_t>(c.na) * c.ns;
    FpxRays r;
    r.vw = reinterpret_cast<float*>(b);
    b += (static_cast<size_t>(c.na) * 4 + 255) & ~static_cast<size_t>(255);
    r.line = reinterpret_cast<FpxLine*>(b);
    b += (static_cast<size_t>(c.na) * sizeof(FpxLine) + 255) & ~static_cast<size_t>(255);
    r.exc = reinterpret_cast<unsigned*>(b);
    b += fpx_exc_bytes(static_cast<long long>(c.na) * c.ns, c.na);
    r.X0 = reinterpret_cast<long long*>(b);
    r.S = reinterpret_cast<long long*>(b + rays * 8);
    r.code = reinterpret_cast<int*>(b + rays * 16);
    r.tie = reinterpret_cast<int*>(b + rays * 20);
    r.views = reinterpret_cast<int*>(b + rays * 24);
    const size_t nviews = 4 * (static_cast<size_t>(c.na) / 4 + 3);
    r.cuts = reinterpret_cast<int*>(b + rays * 24 + nviews * 4);
    const size_t off = (rays * 24 + nviews * 4 + (static_cast<size_t>(c.ctas) + 2) * 4 + 63) &
                       ~static_cast<size_t>(63);
    r.nties = reinterpret_cast<int*>(b + off);
    r.ties = reinterpret_cast<FpxTie*>(b + off + 64);
    return r;
}

// Carves the tables out of `scratch` (256-byte aligned), after the transposed image.
FpxRays fpx_rays(void* scratch, const FpxConst& c, float** imgT)
{
    unsigned char* b = static_cast<unsigned char*>(scratch);
    *imgT = reinterpret_cast<float*>(b);
    b += (static_cast<size_t>(c.total) * sizeof(float) + 255) & ~static_cast<size_t>(255);
    return fpx_tables(b, c);
}

// Ray set-up (and, when imgT_src is given, the transposed copy of it into
// imgT) in one launch, set-up blocks first.
int launch_fpx_setup(const FpxConst& c, const FpxRays& r, const double* sc, const double* bo, const int* usex,
                     const float* img, float* imgT, int batch, cudaStream_t stream)
{
    cudaError_t e = cudaMemsetAsync(r.nties, 0, sizeof(int), stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(r.exc, 0, fpx_exc_bytes(static_cast<long long>(c.na) * c.ns, c.na), stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d: %s", cudaGetErrorString(e));
    const long long rays = static_cast<long long>(c.na) * c.ns;
    const unsigned blocks = static_cast<unsigned>(
        std::min<long long>(div_up(rays, kFpxSetupThreads), 8ll * c.sms));
    const unsigned long long tblocks =
        img ? static_cast<unsigned long long>(div_up(c.n, 32)) * div_up(c.n, 32) * batch : 0ull;
    if (blocks + tblocks > 0x7FFFFFFFull) return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: batch too large");
    fpx_setup<<<static_cast<unsigned>(blocks + tblocks), kFpxSetupThreads, 0, stream>>>(
        bo, usex, sc, c, r, static_cast<int>(blocks), img, imgT);
    return check_launch("fp_par_2d set-up");
}

using FpxKernel = void (*)(const float*, float*, float*, FpxConst, FpxRays, unsigned long long*,
                           unsigned long long);

FpxKernel fpx_kernel(const FpxConst& c, size_t smem, cudaError_t* e)
{
    const FpxKernel k = c.band % 16 == 0 ? fp_proj_f32<16> : (c.band % 8 == 0 ? fp_proj_f32<8> : fp_proj_f32<2>);
    *e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    return k;
}

// The projector on an existing transposed copy imgT.
int launch_fpx_proj(const FpxConst& c, size_t smem, const FpxRays& r, const float* img, float* imgT,
                    float* proj, int batch, cudaStream_t stream)
{
    cudaError_t e;
    const FpxKernel kern = fpx_kernel(c, smem, &e);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
    kern<<<dim3(c.ctas, batch), kFpxThreads, smem, stream>>>(img, imgT, proj, c, r, nullptr, 0ull);
    return check_launch("fp_par_2d");
}

// Whether one image's projector can make its own transposed copy: a
// cooperative launch (every CTA resident at once, so the column-marching
// CTAs may wait for the others' tiles).
bool fpx_fusable(const FpxConst& c, size_t smem)
{
    int dev = 0, coop = 0, per_sm = 0;
    cudaError_t e;
    const FpxKernel kern = fpx_kernel(c, smem, &e);
    if (e != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFpxThreads, smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return static_cast<long long>(per_sm) * c.sms >= c.ctas;
}

// One image with the fused transposed copy: count `tsync` reaches ttarget
// once every CTA has written its tiles of imgT.
int launch_fpx_proj_fused(const FpxConst& c, size_t smem, const FpxRays& r, const float* img, float* imgT,
                          float* proj, unsigned long long* tsync, unsigned long long ttarget,
                          cudaStream_t stream)
{
    cudaError_t e;
    const FpxKernel kern = fpx_kernel(c, smem, &e);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
    FpxConst cc = c;
    FpxRays rr = r;
    void* args[] = {const_cast<float**>(&img), &imgT, &proj, &cc, &rr, &tsync, &ttarget};
    e = cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(c.ctas, 1), dim3(kFpxThreads),
                                    args, smem, stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d (cooperative): %s", cudaGetErrorString(e));
    return check_launch("fp_par_2d");
}

// Transposed copy, ray set-up and the projector, in stream order, on `scratch`.
int launch_fpx(const FpxConst& c, size_t smem, void* scratch, const float* img, float* proj,
               const double* sc, const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    float* imgT = nullptr;
    const FpxRays r = fpx_rays(scratch, c, &imgT);
    int st = launch_fpx_setup(c, r, sc, bo, usex, img, imgT, batch, stream);
    if (st) return st;
    return launch_fpx_proj(c, smem, r, img, imgT, proj, batch, stream);
}

template <typename T>
int fp_forward(const ctr_par_param* p, const T* img, T* proj, const double* sc,
               const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, img, proj, sc, bo, usex, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        FpxConst c;
        size_t smem = 0;
        if (fpx_const(p, img, batch, &c, &smem)) {
            // the transposed image and the per-call ray tables live in stream-ordered scratch
            void* scratch = nullptr;
            const size_t bytes = fpx_scratch_bytes(c);
            cudaError_t e = cudaMallocAsync(&scratch, bytes, stream);
            if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d scratch: %s", cudaGetErrorString(e));
            st = launch_fpx(c, smem, scratch, img, proj, sc, bo, usex, batch, stream);
            cudaFreeAsync(scratch, stream);
            return st;
        }
        // fallback: image bands staged with plain loads
        FpConst c2 = fp_const(p);
        c2.views = std::max(1, std::min(4, kFpThreads * kFpMaxRays / static_cast<int>(p->ns)));
        if (c2.views * static_cast<long long>(p->ns) > kFpThreads * kFpMaxRays)
            return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: ns=%u exceeds %d channels", p->ns,
                        kFpThreads * kFpMaxRays);
        const int len = std::max(p->nx, p->ny) + 1;
        c2.band = std::max(1, std::min(32, 16384 / len));
        const size_t smem2 = sizeof(float) * static_cast<size_t>(c2.band) * len;
        cudaError_t e = cudaFuncSetAttribute(fp_band_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem2));
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
        dim3 grid(div_up(p->na, c2.views), batch);
        fp_band_f32<<<grid, kFpThreads, smem2, stream>>>(img, proj, sc, bo, usex, c2);
    } else {
        dim3 grid(div_up(p->ns, kFp64Threads), p->na, batch);
        fp_ray_kernel<T><<<grid, kFp64Threads, 0, stream>>>(img, proj, sc, bo, usex, p->ns, p->na,
                                                            p->nx, p->ny, p->dx, p->dy,
                                                            static_cast<size_t>(p->nx) * p->ny,
                                                            static_cast<size_t>(p->ns) * p->na);
    }
    return check_launch("fp_par_2d");
}

// The gather over a batch: CTAs of IMG images, the batch's remainder one image per CTA.
template <int ROWS, int IMG>
void fp_adj_launch(const float* proj, float* img, const long long* B, const AdjView* V, const AdjWin* W,
                   const double* pos, const FpConst& c, int tiles_x, int tiles_y, int batch, int segs,
                   int seg_len, float* part, cudaStream_t stream)
{
    constexpr size_t smem = sizeof(float) * kFaViews * FaShape<ROWS>::WIN * 2 * IMG;
    constexpr size_t smem1 = sizeof(float) * kFaViews * FaShape<ROWS>::WIN * 2;
    if (smem > 48 * 1024)  // above the default limit (set per call: the current device's)
        cudaFuncSetAttribute(fp_adj_f32<ROWS, IMG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    const int groups = batch / IMG, zmax = 65535 / segs;  // grid z = groups x segments
    for (int g0 = 0; g0 < groups; g0 += zmax)
        fp_adj_f32<ROWS, IMG><<<dim3(tiles_x, tiles_y, std::min(zmax, groups - g0) * segs), 256, smem, stream>>>(
            proj, img, B, V, W, pos, c, g0 * IMG, segs, seg_len, part, batch);
    if constexpr (IMG > 1) {
        const int rest = batch - groups * IMG;
        if (rest > 0)
            fp_adj_f32<ROWS, 1><<<dim3(tiles_x, tiles_y, rest * segs), 256, smem1, stream>>>(
                proj, img, B, V, W, pos, c, groups * IMG, segs, seg_len, part, batch);
    }
}

template <typename T>
int fp_adjoint(const ctr_par_param* p, const T* proj, T* img, const double* w,
               const double* pos, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, proj, img, w, pos, usex, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        FpConst c = fp_const(p);
        // 32 x 64 tiles, two images per CTA (measured against 32 x 32 tiles
        // and one or four images per CTA at 512^2 x 720 views, batch 1 and 16)
        constexpr int kRows = 8, kImg = 2;
        const int ty = FaShape<kRows>::TY, win = FaShape<kRows>::WIN;
        const int tiles_x = div_up(p->nx, kFaTileX), tiles_y = div_up(p->ny, ty);
        const size_t ntiles = static_cast<size_t>(tiles_x) * tiles_y;
        // View segments per tile: enough CTAs for one image to fill the GPU
        // (3 per SM).  A function of the geometry and device only, so an image's
        // sums are the same in any batch.
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int segs = static_cast<int>(std::max<size_t>(1, std::min<size_t>(8, 3ull * sms / ntiles)));
        const int seg_len = div_up(div_up(static_cast<int>(p->na), segs), kFaViews) * kFaViews;
        segs = div_up(static_cast<int>(p->na), seg_len);
        // tables of the call: fixed-point begin per (view, line), AdjView per
        // view, AdjWin per (view, tile); the segments' partial images
        const size_t nb = sizeof(long long) * p->na * static_cast<size_t>(p->nx);
        const size_t nv = sizeof(AdjView) * p->na;
        const size_t nw = sizeof(AdjWin) * p->na * ntiles;
        const size_t part_at = (nb + nv + nw + 255) / 256 * 256;
        const size_t npart = segs > 1 ? sizeof(float) * segs * batch * c.img_stride : 0;
        void* scratch = nullptr;
        cudaError_t e = cudaMallocAsync(&scratch, part_at + npart, stream);
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d_grad scratch: %s", cudaGetErrorString(e));
        long long* B = static_cast<long long*>(scratch);
        AdjView* V = reinterpret_cast<AdjView*>(static_cast<char*>(scratch) + nb);
        AdjWin* W = reinterpret_cast<AdjWin*>(static_cast<char*>(scratch) + nb + nv);
        float* part = segs > 1 ? reinterpret_cast<float*>(static_cast<char*>(scratch) + part_at) : nullptr;
        fp_adj_prep<<<div_up(static_cast<unsigned long long>(p->na) * p->nx, 256), 256, 0, stream>>>(
            w, pos, usex, B, V, p->na, p->nx);
        fp_adj_windows<<<div_up(static_cast<unsigned long long>(p->na) * std::max(tiles_x, tiles_y) * 32, 256),
                         256, 0, stream>>>(B, V, W, p->na, p->nx, tiles_x, tiles_y, ty, win);
        fp_adj_launch<kRows, kImg>(proj, img, B, V, W, pos, c, tiles_x, tiles_y, batch, segs, seg_len, part,
                                   stream);
        if (segs > 1) {
            const size_t count = static_cast<size_t>(batch) * c.img_stride;
            const bool vec = count % 4 == 0 && reinterpret_cast<uintptr_t>(img) % 16 == 0;
            const unsigned blocks = static_cast<unsigned>(
                std::min<size_t>(div_up(vec ? count / 4 : count, 256), 8ull * sms));
            fp_adj_reduce<<<blocks, 256, 0, stream>>>(part, img, count, segs, vec);
        }
        const unsigned nborder = p->nx == 1 ? 1u : 4u * p->nx - 4u;
        fp_adj_border_f32<<<dim3(nborder, div_up(batch, kFbImg)), 128, 0, stream>>>(proj, img, B, V, pos, c,
                                                                                  batch);
        cudaFreeAsync(scratch, stream);  // after every kernel that reads the tables
    } else {
        dim3 grid(div_up(p->nx, 32), div_up(p->ny, 8), batch);
        fp_adj_kernel<T><<<grid, dim3(32, 8), 0, stream>>>(proj, img, w, pos, usex, p->ns, p->na,
                                                           p->nx, p->ny,
                                                           static_cast<size_t>(p->ns) * p->na,
                                                           static_cast<size_t>(p->nx) * p->ny);
    }
    return check_launch("fp_par_2d_grad");
}

// ---- allocation-free FP32 forward projection ---------------------------------
// For callers that must not allocate device memory inside a call: a host
// framework that hands out all device memory itself (its own pool, a fixed
// arena), or a real-time loop that cannot wait on the allocator.  The
// projector's scratch (the transposed image, 4 bytes a pixel of the batch, and
// its per-call ray tables, 24 bytes a ray plus ~400 KB) lives in this fixed
// file-scope array instead of stream-ordered scratch: 16 MiB, e.g. 720 views x
// 729 bins with up to 3 images of 512^2.  Every call writes all of the scratch
// it reads (the tie counter by a memset), so nothing in the array has to start
// at zero.
// All calls on a device share the one array: calls ordered on one stream are
// safe, calls that can overlap (two streams, two host threads without
// ordering) race on it and give wrong results.
constexpr long long kFpNoAllocBytes = 16ll << 20;
static __device__ __align__(256) unsigned char g_fp_noalloc_scratch[kFpNoAllocBytes];

// The array's device address in the current context (cudaGetSymbolAddress on
// every call: cheap once the module is loaded, and never stale after a device
// reset or under another context; the first call in a context loads the module).
int noalloc_scratch(void** out)
{
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_fp_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
        return fail(CTR_ERR_CUDA, "fp_par_2d_f32_noalloc scratch address: %s", cudaGetErrorString(e));
    *out = ptr;
    return CTR_OK;
}

int fp_forward_noalloc(const ctr_par_param* p, const float* img, float* proj, const double* sc,
                       const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, img, proj, sc, bo, usex, batch);
    if (st) return st;
    FpxConst c;
    size_t smem = 0;
    if (!fpx_const(p, img, batch, &c, &smem))
        return fail(CTR_ERR_UNSUPPORTED,
                    "fp_par_2d_f32_noalloc: needs a 16-byte aligned img and nx <= 8192");
    const size_t need = fpx_scratch_bytes(c);
    if (need > static_cast<size_t>(kFpNoAllocBytes))
        return fail(CTR_ERR_UNSUPPORTED,
                    "fp_par_2d_f32_noalloc: %zu bytes of scratch (24 per ray, 4 per image pixel) "
                    "exceed its fixed 16 MiB; split the batch or call ctr_fp_par_2d_f32",
                    need);
    void* scratch = nullptr;
    st = noalloc_scratch(&scratch);
    if (st) return st;
    return launch_fpx(c, smem, scratch, img, proj, sc, bo, usex, batch, stream);
}

}  // namespace
}  // namespace ctr

// A per-geometry plan of the FP32 ray-driven projector: the ray tables (fixed-
// point start and step, exact sample range and class of every ray, the
// reference's decisions for its tie rays, view lists, CTA cut and view
// weights) are built once from the caller's tables; a call then runs the
// transposed copy and the projector only.
struct ctr_fp_plan {
    int device = 0;
    int max_batch = 0;
    ctr::FpxConst c{};
    size_t smem = 0;
    void* tables = nullptr;
    float* imgT = nullptr;
    ctr::FpxRays r{};
    bool fused = false;                  // one-image calls make their own transposed copy
    unsigned long long* tsync = nullptr; // the fused copy's CTA count (never reset)
    unsigned long long calls = 0;        // fused calls so far: count target = calls * ctas
    ~ctr_fp_plan()
    {
        if (tables) cudaFree(tables);
        if (imgT) cudaFree(imgT);
        if (tsync) cudaFree(tsync);
    }
};

using namespace ctr;

extern "C" {

int ctr_fp_par_2d_plan_create(const ctr_par_param* p, const double* sincostbl, const double* beginoffset,
                              const int* usex, int max_batch, ctr_fp_plan** plan, cudaStream_t stream)
{
    if (!plan) return fail(CTR_ERR_INVALID_ARG, "null plan pointer");
    *plan = nullptr;
    int st = check_fp(p, sincostbl, beginoffset, sincostbl, beginoffset, usex, max_batch);
    if (st) return st;
    FpxConst c;
    size_t smem = 0;
    alignas(16) static const float probe[4] = {};  // the plan checks the caller's image per call
    if (!fpx_const(p, probe, max_batch, &c, &smem))
        return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d plan: needs nx <= 8192 and fewer than 2^30 ray slots");
    auto P = std::make_unique<ctr_fp_plan>();
    cudaGetDevice(&P->device);
    P->max_batch = max_batch;
    P->c = c;
    P->smem = smem;
    const size_t tbytes = fpx_table_bytes(static_cast<long long>(c.na) * c.ns, c.na, c.ctas);
    const size_t ibytes = static_cast<size_t>(max_batch) * c.n * c.n * sizeof(float);
    if (cudaMalloc(&P->tables, tbytes) != cudaSuccess || cudaMalloc(&P->imgT, ibytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(CTR_ERR_CUDA, "fp_par_2d plan: %zu + %zu bytes", tbytes, ibytes);
    }
    P->r = fpx_tables(static_cast<unsigned char*>(P->tables), c);
    P->fused = fpx_fusable(c, smem);
    if (P->fused && (cudaMalloc(&P->tsync, sizeof(unsigned long long)) != cudaSuccess ||
                     cudaMemsetAsync(P->tsync, 0, sizeof(unsigned long long), stream) != cudaSuccess)) {
        cudaGetLastError();
        return fail(CTR_ERR_CUDA, "fp_par_2d plan: sync counter");
    }
    st = launch_fpx_setup(c, P->r, sincostbl, beginoffset, usex, nullptr, nullptr, 1, stream);
    if (st) return st;
    const cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d plan set-up: %s", cudaGetErrorString(e));
    *plan = P.release();
    return CTR_OK;
}

int ctr_fp_par_2d_plan_run(ctr_fp_plan* plan, const float* img, float* proj, int batch, cudaStream_t stream)
{
    if (!plan || !img || !proj) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != plan->device) return fail(CTR_ERR_INVALID_ARG, "plan made on device %d, current %d", plan->device, dev);
    if (batch > plan->max_batch) return fail(CTR_ERR_INVALID_ARG, "batch %d > the plan's %d", batch, plan->max_batch);
    if (reinterpret_cast<uintptr_t>(img) % 16 != 0)
        return fail(CTR_ERR_INVALID_ARG, "fp_par_2d plan: img must be 16-byte aligned");
    FpxConst c = plan->c;
    c.total = static_cast<long long>(batch) * c.n * c.n;
    c.total4 = c.total & ~3ll;
    if (batch == 1 && plan->fused) {
        ++plan->calls;
        return launch_fpx_proj_fused(c, plan->smem, plan->r, img, plan->imgT, proj, plan->tsync,
                                     plan->calls * static_cast<unsigned long long>(c.ctas), stream);
    }
    const unsigned long long tiles = static_cast<unsigned long long>(div_up(c.n, 32)) * div_up(c.n, 32) * batch;
    if (tiles > 0x7FFFFFFFull) return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: batch too large");
    fpx_transpose<<<static_cast<unsigned>(tiles), kFpxSetupThreads, 0, stream>>>(img, plan->imgT, c.n);
    st = check_launch("fp_par_2d transposed copy");
    if (st) return st;
    return launch_fpx_proj(c, plan->smem, plan->r, img, plan->imgT, proj, batch, stream);
}

int ctr_fp_par_2d_plan_destroy(ctr_fp_plan* plan)
{
    delete plan;
    return CTR_OK;
}

int ctr_fp_par_2d_f32(const ctr_par_param* p, const float* img, float* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream)
{
    return fp_forward<float>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_f64(const ctr_par_param* p, const double* img, double* proj,
                      const double* sincostbl, const double* beginoffset, const int* usex,
                      int batch, cudaStream_t stream)
{
    return fp_forward<double>(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}
int ctr_fp_par_2d_grad_f32(const ctr_par_param* p, const float* proj, float* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream)
{
    return fp_adjoint<float>(p, proj, img, weights, pos, usex, batch, stream);
}
int ctr_fp_par_2d_grad_f64(const ctr_par_param* p, const double* proj, double* img,
                           const double* weights, const double* pos, const int* usex,
                           int batch, cudaStream_t stream)
{
    return fp_adjoint<double>(p, proj, img, weights, pos, usex, batch, stream);
}
int ctr_fp_par_2d_f32_noalloc(const ctr_par_param* p, const float* img, float* proj,
                              const double* sincostbl, const double* beginoffset, const int* usex,
                              int batch, cudaStream_t stream)
{
    return fp_forward_noalloc(p, img, proj, sincostbl, beginoffset, usex, batch, stream);
}

}  // extern "C"

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
#include <mutex>
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
// a strided order (slot_octet), so a contiguous range of slots mixes long
// central rays and short edge rays.  Each class gets CTAs in proportion to its
// views and cuts its slots into equal ranges, and a CTA deals its slots, sorted
// by their exact sample counts, to its warps in snake order.  A round holds up
// to kFpxRound slots (one more round streams the image again; rare).
//
// Pipeline: a producer lane copies band t (one contiguous range of the staged
// row-major array, one TMA bulk copy) into stage t % 3 once every consumer
// warp has released that stage, so warps drift up to two bands apart instead
// of meeting at a CTA barrier per band.  Within a band a sample costs one
// 64-bit add, the address, two shared loads, the fraction and two FP32
// operations: the position's high word indexes the stage directly
// (S2 = S + n * 2^32 steps one row down).
//
// Ties: a ray whose end sample lies within a hair of the image border (where
// the fixed-point rule might differ from the reference's accumulated FP64
// one) streams only its certain samples; the set-up decides its few border
// samples by the reference's accumulation (acc_advance) and the ray's lane
// adds the ones found inside, read from global memory, before writing.
constexpr int kFpxWarps = 9;                         // consumer warps
constexpr int kFpxThreads = (kFpxWarps + 1) * 32;    // + one producer warp
constexpr int kFpxSlots = 8;                         // ray slots per consumer lane and round
constexpr int kFpxRound = kFpxWarps * kFpxSlots;     // slots per round
constexpr int kFpxStages = 3;
constexpr int kFpxStageFloats = 8192;                // nominal stage: 32 KB
constexpr int kFpxEmpty = 3 << 30;                   // ray code of a ray with no sample
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
};

// Global tie entry (a ray the fixed-point rule could not settle).
struct FpxTie {
    int namb;
    unsigned in;  // bit a: amb[a] is inside by the reference's accumulated rule
    int amb[4];   // ambiguous samples next to the certain range
};

// The per-call tables (scratch) written by fpx_setup.
struct FpxRays {
    long long* X0;   // [na*ns] 32.32 position of sample 0
    long long* S;    // [na*ns] 32.32 step
    int* code;       // [na*ns] k0 | k1 << 15 | class << 30, or kFpxEmpty
    int* tie;        // [na*ns] index into ties, or -1
    int* views;      // [4 * (quads + 2)] views of class 0, then of class 1, -1 padded to quads
    int* cuts;       // [ctas + 1] first slot of every CTA; cuts[ctas + 1] = CTAs of class 0
    FpxTie* ties;    // [kFpxMaxTies]
    int* nties;      // count (zeroed before fpx_setup)
};

__host__ __device__ inline size_t fpx_table_bytes(long long rays, int na, int ctas)
{
    const size_t r = static_cast<size_t>(rays);
    const size_t views = 4 * (static_cast<size_t>(na) / 4 + 3);
    return ((r * 24 + views * 4 + (static_cast<size_t>(ctas) + 2) * 4 + 63) & ~static_cast<size_t>(63)) +
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

// ---- set-up kernel: every ray once; block 0 the class lists and CTA cut ------
// Blocks from `setup_blocks` on transpose the images instead (32 x 32 tiles):
// the two jobs are independent, and the transpose blocks fill the SMs left idle
// while the few tie rays of the set-up walk the reference's accumulation.
__global__ void __launch_bounds__(kFpxSetupThreads)
    fpx_setup(const double* __restrict__ bo, const int* __restrict__ usex, const FpxConst c,
              const FpxRays r, int setup_blocks, const float* __restrict__ img, float* __restrict__ imgT)
{
    __shared__ int s_chunk[2049];  // block 0: row-marching views before each chunk of 32
    const int tid = threadIdx.x;
    if (static_cast<int>(blockIdx.x) >= setup_blocks) {
        // imgT[b][x][y] = img[b][y][x]
        float (*t)[33] = reinterpret_cast<float (*)[33]>(s_chunk);  // 32 x 33 floats
        const int n = c.n, tiles = (n + 31) / 32;
        const int tb = static_cast<int>(blockIdx.x) - setup_blocks;
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
        return;
    }
    if (blockIdx.x == 0) {
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
        // CTAs per class in proportion to its views, each class cut into equal
        // slot ranges (a view costs about the same at every angle: fewer samples
        // at 45 degrees, but longer shared-memory and lane waits)
        int G0 = 0;
        if (N0 > 0) G0 = N1 > 0 ? static_cast<int>(rintf(static_cast<float>(c.ctas) * N0 / c.na)) : c.ctas;
        if (N0 > 0 && N1 > 0) G0 = max(1, min(c.ctas - 1, G0));
        const int G1 = c.ctas - G0;
        for (int i = tid; i <= c.ctas; i += kFpxSetupThreads) {
            const bool cls1 = i > G0 || (i == G0 && G0 == 0);
            const long long gi = cls1 ? i - G0 : i, G = cls1 ? G1 : G0;
            const long long s0 = static_cast<long long>(cls1 ? Q0 : 0) * c.octets;
            const long long ns_ = static_cast<long long>(cls1 ? Q1 : Q0) * c.octets;
            r.cuts[i] = static_cast<int>(s0 + (G > 0 ? (gi * ns_) / G : 0));
        }
        if (tid == 0) r.cuts[c.ctas + 1] = G0;
    }
    const int rays = c.na * c.ns;
    for (int ray = blockIdx.x * kFpxSetupThreads + tid; ray < rays; ray += setup_blocks * kFpxSetupThreads) {
        const int ia = ray / c.ns;
        const double begin = bo[2 * static_cast<size_t>(ray)], step = bo[2 * static_cast<size_t>(ray) + 1];
        long long X0 = 0, S = 0;
        int k0, k1, tie = -1;
        if (!ray_fixed(begin, step, c.n, &X0, &S, &k0, &k1)) {
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
        const int cls = usex[ia] != 0 ? 0 : 1;
        r.X0[ray] = X0;
        r.S[ray] = S;
        r.code[ray] = k0 <= k1 ? (k0 | (k1 << 15) | (cls << 30)) : kFpxEmpty;
        r.tie[ray] = tie;
    }
}

__global__ void __launch_bounds__(kFpxThreads, 2)
    fp_proj_f32(const float* __restrict__ img, const float* __restrict__ imgT,
                float* __restrict__ proj, const double* __restrict__ sincos,
                const int* __restrict__ usex, const FpxConst c, const FpxRays r)
{
    extern __shared__ __align__(128) unsigned char fpx_dyn[];
    float* stage = reinterpret_cast<float*>(fpx_dyn + ((128u - (smem_u32(fpx_dyn) & 127u)) & 127u));
    __shared__ __align__(8) unsigned long long s_full[kFpxStages], s_empty[kFpxStages];
    __shared__ int s_work[kFpxRound];
    __shared__ int s_assign[kFpxWarps][kFpxSlots];  // slot of the round, or -1
    __shared__ int s_abort;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n = c.n;
    const long long item0 = static_cast<long long>(blockIdx.y) * n * n;
    const float* I = img + item0;
    const int q_lo = r.cuts[blockIdx.x], q_hi = r.cuts[blockIdx.x + 1];
    const bool cls1 = static_cast<int>(blockIdx.x) >= r.cuts[c.ctas + 1];
    const float* src = cls1 ? imgT : img;  // the staged array: rows are the marched lines
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < kFpxStages; ++s) {
            mbar_init(smem_u32(&s_full[s]), 1);
            mbar_init(smem_u32(&s_empty[s]), kFpxWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }

    int g = 0;  // band instances so far (producer and consumers count alike)
    for (int base = q_lo; base < q_hi; base += kFpxRound) {
        const int m = min(kFpxRound, q_hi - base);
        for (int i = tid; i < kFpxRound; i += kFpxThreads) (&s_assign[0][0])[i] = -1;
        // ---- sample counts of the round's slots
        if (warp < kFpxWarps) {
            for (int t = warp; t < m; t += kFpxWarps) {
                int ia, is, cnt = 0;
                slot_ray(static_cast<unsigned>(base + t), lane, c, r.views, &ia, &is);
                if (ia >= 0 && is < c.ns) {
                    const int code = r.code[ia * c.ns + is];
                    if (code != kFpxEmpty) cnt = ((code >> 15) & 0x7FFF) - (code & 0x7FFF) + 1;
                }
                const unsigned tot = __reduce_add_sync(0xffffffffu, static_cast<unsigned>(cnt));
                if (lane == 0) s_work[t] = static_cast<int>(tot);
            }
        }
        __syncthreads();
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
        // zero the stages: the few slack elements past a band read as finite
        for (int i = tid; i < kFpxStages * c.stage_floats; i += kFpxThreads) stage[i] = 0.0f;
        __syncthreads();

        if (warp == kFpxWarps) {
            // ---- producer: one lane issues every band
            if (lane == 0) {
                bool alive = true;
                int g1 = g;
                for (int t = 0; t < c.nbands; ++t, ++g1) {
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
                    slot_ray(static_cast<unsigned>(base + t), lane, c, r.views, &ia, &is);
                    if (ia >= 0 && is < c.ns) {
                        const int ray = ia * c.ns + is;
                        code[j] = r.code[ray];
                        X0[j] = r.X0[ray];
                        S[j] = r.S[ray];
                    }
                }
            }
            int g1 = g;
            bool alive = true;
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
                    const int cj = code[j];
                    if (cj == kFpxEmpty) continue;
                    const int ka = max(cj & 0x7FFF, b0), kb = min((cj >> 15) & 0x7FFF, b1);
                    if (ka > kb) continue;
                    long long x = X0[j] + static_cast<long long>(ka) * S[j] +
                                  (static_cast<long long>((ka - b0) * n) << 32);
                    const long long S2 = S[j] + (static_cast<long long>(n) << 32);
                    float a = 0.0f, b = 0.0f;  // this band's partial sums (blocked summation)
#pragma unroll 4
                    for (int k = ka; k <= kb; ++k) {
                        const float* p = bb + static_cast<int>(x >> 32);
                        const float p0 = p[0], p1 = p[1];
                        a += p0;
                        b = fmaf(frac_of(x), p1 - p0, b);
                        x += S2;
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
                slot_ray(static_cast<unsigned>(base + t), lane, c, r.views, &ia, &is);
                if (ia < 0 || is >= c.ns) continue;
                float v = sum[j];
                const int gi = r.tie[ia * c.ns + is];
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
                const float dw = cls1 ? c.dx / fabsf(dbl2flt(sincos[2 * ia]))
                                      : c.dy / fabsf(dbl2flt(sincos[2 * ia + 1]));
                proj[blockIdx.y * c.proj_stride + static_cast<size_t>(ia) * c.ns + is] = v * dw;
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
// clamp at 0 is the footprint's edge).  fp_adj_prep converts the caller's
// positions to 32.32 fixed point once per call; fp_adj_f32 stages, per block
// of views, the channel window of its 32 x 64 tile as zero-padded (p[i], p[i+1]) pairs in
// shared memory, so such a pixel-view is one 8-byte shared load and a few
// FMAs; positions advance by 64-bit adds.  It computes every pixel that way.
// Pixels on the image border have one-sided footprints (channels on the
// neighbour's side only); fp_adj_border_f32 then recomputes those 4n - 4
// pixels exactly (one warp each) and overwrites them.  Views with |offset| > 1 or a window
// wider than the staged one take the exact per-pixel path in both kernels.
constexpr int kFaViews = 16;
constexpr int kFaRows = 8;                 // pixels per thread (one column)
constexpr int kFaTileX = 32, kFaTileY = 8 * kFaRows;  // 32 x 64 tile, 256 threads
constexpr int kFaLines = kFaTileY;         // lines of a tile: rows (64) or columns (32)
constexpr int kFaWin = 128;                // staged channel pairs per view
// Units of 2^-32 channel within which a border pixel's position counts as on a
// channel: the fixed-point position is within 0.5 + 0.5*along units of the
// reference's FP64 one (along < 8192).
constexpr unsigned kFaTie = 8192;

// 32.32 fixed point of a table value: integer conversion where exact, FP64 beyond.
__device__ __forceinline__ long long fix32_any(double v)
{
    return ((double_bits(v) >> 52) & 0x7FF) < 1043 ? fix32(v) : llrint(v * kTwo32);
}

// The reference grad's tap sum for one pixel-view: MID = the pixel's position
// (fixed point), O1 = the view's offset, `along` = the pixel's index along its
// line, pp = the caller's (begin, offset) of the pixel's line.  A border pixel's
// footprint is one-sided (toward the neighbour pixel); its end channel is
// decided from the fixed-point fraction or, when mid lies within kFaTie units
// of a channel, in FP64 exactly as the reference does.
__device__ __forceinline__ float adj_tap_exact(const float* __restrict__ row, long long MID, long long O1,
                                               float inv, bool two, int along, int n, int ns,
                                               const double* __restrict__ pp)
{
    const int mi = static_cast<int>(MID >> 32);
    const float mf = frac_of(MID);
    const bool border = along == 0 || along == n - 1;
    const unsigned frac_bits = static_cast<unsigned>(MID);
    const bool tie = border && (n == 1 || frac_bits < kFaTie || frac_bits > 0u - kFaTie);
    if (two && !tie) {
        float w0 = fmaxf(fmaf(-mf, inv, 1.0f), 0.0f);
        float w1 = fmaxf(fmaf(mf, inv, 1.0f - inv), 0.0f);
        if (border) {
            const bool ge = (along == 0) != (O1 < 0);  // footprint [mid, mid + |o|]
            if (ge) w0 = 0.0f;
            else w1 = 0.0f;
        }
        const float p0 = static_cast<unsigned>(mi) < static_cast<unsigned>(ns) ? __ldg(row + mi) : 0.0f;
        const float p1 = static_cast<unsigned>(mi + 1) < static_cast<unsigned>(ns) ? __ldg(row + mi + 1) : 0.0f;
        return fmaf(w0, p0, w1 * p1);
    }
    long long L = along == 0 ? MID : MID - O1;
    long long R = along == n - 1 ? MID : MID + O1;
    if (L > R) {
        const long long t = L;
        L = R;
        R = t;
    }
    int lo = max(static_cast<int>((L + 0xFFFFFFFFll) >> 32), 0);
    int hi = min(static_cast<int>(R >> 32), ns - 1);
    if (border) {
        // the end channel sits at the pixel itself with weight ~1: the range
        // is decided in FP64 as the reference does (mid = begin + offset*along)
        const double off = pp[1];
        const double mid = __dadd_rn(pp[0], __dmul_rn(off, static_cast<double>(along)));
        double left = along == 0 ? mid : __dsub_rn(mid, off);
        double right = along == n - 1 ? mid : __dadd_rn(mid, off);
        if (left > right) {
            const double t = left;
            left = right;
            right = t;
        }
        lo = static_cast<int>(fmax(ceil(left), 0.0));
        hi = static_cast<int>(fmin(floor(right), static_cast<double>(ns - 1)));
    }
    float part = 0.0f;
    for (int is = lo; is <= hi; ++is) {
        const float d = fabsf(mf - static_cast<float>(is - mi));
        part = fmaf(fmaf(-d, inv, 1.0f), __ldg(row + is), part);
    }
    return part;
}

__device__ __forceinline__ float2 lds_pair(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

// Per-view constants of the adjoint, from the caller's grad-prep tables.
struct AdjView {
    long long O1;  // offset, 32.32 fixed point
    float inv;     // 1 / |offset|
    float w;       // view weight
    int ux;        // lines are rows
    int two;       // |offset| <= 1
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

__global__ void __launch_bounds__(256, 3)
    fp_adj_f32(const float* __restrict__ proj, float* __restrict__ img, const long long* __restrict__ B,
               const AdjView* __restrict__ V, const double* __restrict__ pos, const FpConst c)
{
    __shared__ long long s_base[kFaViews][kFaLines];
    __shared__ AdjView s_v[kFaViews];
    __shared__ int s_lo[kFaViews], s_hi[kFaViews];
    __shared__ __align__(16) float2 s_pair[kFaViews][kFaWin];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx0 = blockIdx.x * kFaTileX, ty0 = blockIdx.y * kFaTileY;
    const int ix = tx0 + lane;
    const float* P = proj + blockIdx.z * c.proj_stride;
    float acc[kFaRows];
#pragma unroll
    for (int r = 0; r < kFaRows; ++r) acc[r] = 0.0f;
    const int n = c.nx;  // == ny
    const int ns = c.ns;

    for (int v0 = 0; v0 < c.na; v0 += kFaViews) {
        const int nv = min(kFaViews, c.na - v0);
        if (threadIdx.x < nv) {
            s_v[threadIdx.x] = V[v0 + threadIdx.x];
            s_lo[threadIdx.x] = INT_MAX;
            s_hi[threadIdx.x] = INT_MIN;
        }
        __syncthreads();
        // line positions of the tile (rows for row-marching views, else
        // columns) and the tile's channel range: for a fixed line the position
        // is linear in `along`, extreme at the tile's first and last along index.
        // Fixed trip count: every load of the block is in flight at once.
#pragma unroll
        for (int it = 0; it < kFaViews * kFaLines / 256; ++it) {
            const int idx = it * 256 + threadIdx.x;
            const int j = idx / kFaLines, l = idx - j * kFaLines;  // a warp's lanes share j
            int lo = INT_MAX, hi = INT_MIN;
            if (j < nv) {
                const AdjView& v = s_v[j];
                if (l < (v.ux ? kFaTileY : kFaTileX)) {
                    const int lin = min((v.ux ? ty0 : tx0) + l, n - 1);
                    const long long b = __ldg(B + static_cast<size_t>(v0 + j) * n + lin);
                    s_base[j][l] = b;
                    const long long m0 = b + static_cast<long long>(v.ux ? tx0 : ty0) * v.O1;
                    const long long m1 = m0 + static_cast<long long>((v.ux ? kFaTileX : kFaTileY) - 1) * v.O1;
                    lo = static_cast<int>((m0 < m1 ? m0 : m1) >> 32);
                    hi = static_cast<int>((m0 < m1 ? m1 : m0) >> 32);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if ((threadIdx.x & 31) == 0 && lo <= hi) {
                atomicMin(&s_lo[j], lo);
                atomicMax(&s_hi[j], hi);
            }
        }
        __syncthreads();
        // staged windows: (p[lo+k], p[lo+k+1]), zero off the detector
#pragma unroll
        for (int it = 0; it < kFaViews * kFaWin / 256; ++it) {
            const int idx = it * 256 + threadIdx.x;
            const int j = idx / kFaWin, k = idx - j * kFaWin;
            if (j < nv && s_v[j].two && s_hi[j] - s_lo[j] + 2 <= kFaWin) {
                const float* row = P + static_cast<size_t>(v0 + j) * ns;
                const int g = s_lo[j] + k;
                const float p0 = static_cast<unsigned>(g) < static_cast<unsigned>(ns) ? __ldg(row + g) : 0.0f;
                const float p1 = static_cast<unsigned>(g + 1) < static_cast<unsigned>(ns) ? __ldg(row + g + 1) : 0.0f;
                s_pair[j][k] = make_float2(p0, p1);
            }
        }
        __syncthreads();
        float blk[kFaRows];  // this view block's partial sums (blocked summation)
#pragma unroll
        for (int r = 0; r < kFaRows; ++r) blk[r] = 0.0f;
        for (int j = 0; j < nv; ++j) {
            const AdjView v = s_v[j];
            const int lo = s_lo[j];
            if (v.two && s_hi[j] - lo + 2 <= kFaWin) {
                const float inv1 = 1.0f - v.inv;
                const unsigned pb = smem_u32(&s_pair[j][0]) - 8u * static_cast<unsigned>(lo);
                if (v.ux) {  // along = ix, line = row
                    const long long A = static_cast<long long>(ix) * v.O1;
#pragma unroll
                    for (int r = 0; r < kFaRows; ++r) {
                        const long long MID = s_base[j][warp * kFaRows + r] + A;
                        const float mf = frac_of(MID);
                        const float2 pv = lds_pair(pb + 8u * static_cast<unsigned>(MID >> 32));
                        const float w0 = __saturatef(fmaf(-mf, v.inv, 1.0f));
                        const float w1 = __saturatef(fmaf(mf, v.inv, inv1));
                        blk[r] = fmaf(fmaf(w0, pv.x, w1 * pv.y), v.w, blk[r]);
                    }
                } else {   // along = row, line = ix
                    long long MID = s_base[j][lane] + static_cast<long long>(ty0 + warp * kFaRows) * v.O1;
#pragma unroll
                    for (int r = 0; r < kFaRows; ++r) {
                        const float mf = frac_of(MID);
                        const float2 pv = lds_pair(pb + 8u * static_cast<unsigned>(MID >> 32));
                        const float w0 = __saturatef(fmaf(-mf, v.inv, 1.0f));
                        const float w1 = __saturatef(fmaf(mf, v.inv, inv1));
                        blk[r] = fmaf(fmaf(w0, pv.x, w1 * pv.y), v.w, blk[r]);
                        MID += v.O1;
                    }
                }
            } else {
                const float* row = P + static_cast<size_t>(v0 + j) * ns;
#pragma unroll
                for (int r = 0; r < kFaRows; ++r) {
                    const int iy = ty0 + warp * kFaRows + r;
                    const int along = v.ux ? ix : iy;
                    const int lin = v.ux ? iy : ix;
                    const long long MID = s_base[j][v.ux ? warp * kFaRows + r : lane] +
                                          static_cast<long long>(along) * v.O1;
                    const double* pp = pos + (static_cast<size_t>(v0 + j) * n + min(lin, n - 1)) * 2;
                    blk[r] = fmaf(adj_tap_exact(row, MID, v.O1, v.inv, v.two != 0, along, n, ns, pp), v.w,
                                  blk[r]);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < kFaRows; ++r) acc[r] += blk[r];
        __syncthreads();
    }
    float* O = img + blockIdx.z * c.img_stride;
#pragma unroll
    for (int r = 0; r < kFaRows; ++r) {
        const int iy = ty0 + warp * kFaRows + r;
        if (ix < c.nx && iy < c.ny) O[static_cast<size_t>(iy) * c.nx + ix] = acc[r];
    }
}

// The 4n - 4 border pixels, exactly, overwriting fp_adj_f32's values: one
// warp per pixel, lane l summing views l, l+32, ..., then a fixed shuffle tree.
__global__ void __launch_bounds__(128)
    fp_adj_border_f32(const float* __restrict__ proj, float* __restrict__ img,
                      const long long* __restrict__ B, const AdjView* __restrict__ V,
                      const double* __restrict__ pos, const FpConst c)
{
    const int n = c.nx, ns = c.ns;
    const int nb = n == 1 ? 1 : 4 * n - 4;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (b >= nb) return;  // warp-uniform
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
    const float* P = proj + blockIdx.y * c.proj_stride;
    float acc = 0.0f;
    for (int ia = lane; ia < c.na; ia += 32) {
        const AdjView v = V[ia];
        const int along = v.ux ? ix : iy, lin = v.ux ? iy : ix;
        const size_t line = static_cast<size_t>(ia) * n + lin;
        const long long MID = __ldg(B + line) + static_cast<long long>(along) * v.O1;
        const float part = adj_tap_exact(P + static_cast<size_t>(ia) * ns, MID, v.O1, v.inv, v.two != 0,
                                         along, n, ns, pos + line * 2);
        acc = fmaf(part, v.w, acc);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) img[blockIdx.y * c.img_stride + static_cast<size_t>(iy) * n + ix] = acc;
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
    // two CTAs an SM; more when the mean CTA would exceed 7/8 of a round
    const long long ctas = std::max<long long>(div_up(slots * 8, kFpxRound * 7), 2 * kSmCount);
    c.ctas = static_cast<int>(std::min<long long>(ctas, slots));
    c.band = std::max(1, std::min(32, kFpxStageFloats / n));
    c.nbands = static_cast<int>(div_up(n, c.band));
    c.stage_floats = (c.band * n + 8 + 31) / 32 * 32;
    c.total = static_cast<long long>(batch) * n * n;
    c.total4 = c.total & ~3ll;
    c.proj_stride = static_cast<size_t>(p->ns) * p->na;
    c.dx = static_cast<float>(p->dx);
    c.dy = static_cast<float>(p->dy);
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

// Carves the tables out of `scratch` (256-byte aligned), after the transposed image.
FpxRays fpx_rays(void* scratch, const FpxConst& c, float** imgT)
{
    const size_t rays = static_cast<size_t>(c.na) * c.ns;
    unsigned char* b = static_cast<unsigned char*>(scratch);
    *imgT = reinterpret_cast<float*>(b);
    b += (static_cast<size_t>(c.total) * sizeof(float) + 255) & ~static_cast<size_t>(255);
    FpxRays r;
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

// Transposed copy, ray set-up and the projector, in stream order, on `scratch`.
int launch_fpx(const FpxConst& c, size_t smem, void* scratch, const float* img, float* proj,
               const double* sc, const double* bo, const int* usex, int batch, cudaStream_t stream)
{
    float* imgT = nullptr;
    const FpxRays r = fpx_rays(scratch, c, &imgT);
    const int n = c.n;
    cudaError_t e = cudaMemsetAsync(r.nties, 0, sizeof(int), stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d: %s", cudaGetErrorString(e));
    const long long rays = static_cast<long long>(c.na) * c.ns;
    const unsigned blocks = static_cast<unsigned>(
        std::min<long long>(div_up(rays, kFpxSetupThreads), 8 * kSmCount));
    const unsigned long long tblocks = static_cast<unsigned long long>(div_up(n, 32)) * div_up(n, 32) * batch;
    if (blocks + tblocks > 0x7FFFFFFFull) return fail(CTR_ERR_UNSUPPORTED, "fp_par_2d: batch too large");
    // ray set-up and the transposed copy in one launch (set-up blocks first)
    fpx_setup<<<static_cast<unsigned>(blocks + tblocks), kFpxSetupThreads, 0, stream>>>(
        bo, usex, c, r, static_cast<int>(blocks), img, imgT);
    int st = check_launch("fp_par_2d set-up");
    if (st) return st;
    e = cudaFuncSetAttribute(fp_proj_f32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp smem: %s", cudaGetErrorString(e));
    fp_proj_f32<<<dim3(c.ctas, batch), kFpxThreads, smem, stream>>>(img, imgT, proj, sc, usex, c, r);
    return check_launch("fp_par_2d");
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

template <typename T>
int fp_adjoint(const ctr_par_param* p, const T* proj, T* img, const double* w,
               const double* pos, const int* usex, int batch, cudaStream_t stream)
{
    int st = check_fp(p, proj, img, w, pos, usex, batch);
    if (st) return st;
    if constexpr (sizeof(T) == 4) {
        FpConst c = fp_const(p);
        // fixed-point tables of the call (int64 per (view, line), AdjView per view)
        const size_t nb = sizeof(long long) * p->na * static_cast<size_t>(p->nx);
        void* scratch = nullptr;
        cudaError_t e = cudaMallocAsync(&scratch, nb + sizeof(AdjView) * p->na, stream);
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fp_par_2d_grad scratch: %s", cudaGetErrorString(e));
        long long* B = static_cast<long long*>(scratch);
        AdjView* V = reinterpret_cast<AdjView*>(static_cast<char*>(scratch) + nb);
        fp_adj_prep<<<div_up(static_cast<unsigned long long>(p->na) * p->nx, 256), 256, 0, stream>>>(
            w, pos, usex, B, V, p->na, p->nx);
        dim3 grid(div_up(p->nx, kFaTileX), div_up(p->ny, kFaTileY), batch);
        fp_adj_f32<<<grid, 256, 0, stream>>>(proj, img, B, V, pos, c);
        const unsigned nborder = p->nx == 1 ? 1u : 4u * p->nx - 4u;
        fp_adj_border_f32<<<dim3(div_up(nborder, 4), batch), 128, 0, stream>>>(proj, img, B, V, pos, c);
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

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// The array's device address on the current device, looked up once per device
// (cudaGetSymbolAddress; the first call on a device does this set-up).
int noalloc_scratch(void** out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(CTR_ERR_DEVICE, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kNoAllocMaxDevices)
        return fail(CTR_ERR_UNSUPPORTED, "device %d >= %d", dev, kNoAllocMaxDevices);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_fp_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(CTR_ERR_CUDA, "fp_par_2d_f32_noalloc scratch address: %s",
                        cudaGetErrorString(e));
        g_noalloc_ptr[dev] = ptr;
    }
    *out = g_noalloc_ptr[dev];
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

using namespace ctr;

extern "C" {

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

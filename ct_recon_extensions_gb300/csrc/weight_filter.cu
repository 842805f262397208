// Fan weighting and ramp filtering (reference src/fan_weighting.cc:19-59,
// src/filter.cc:67-124).
//
// Fan weighting is an HBM-bound diagonal scaling: a CTA computes the FP64
// weights of its channels once and streams a block of rows, multiplying in
// FP64 exactly as the reference does (results are bit-identical to its CPU
// code for both T).
//
// The ramp filter is a linear (zero-padded) convolution with 2ns+1 taps.  A
// CTA stages kRows rows and the taps in shared memory; each thread produces
// one output column for all staged rows, so a tap load is shared by kRows
// multiply-adds.  The reference kernels have zero even taps (k != 0); when
// the caller's table has that structure (checked in-kernel) only the odd
// taps are visited.
//
// FP32 accuracy: the ramp taps sum to almost zero, so on a smooth sinogram
// the output is a small difference of large partial sums.  The FP32 kernel
// therefore accumulates h[o-j] (x[j] - c) with c a value of the row near the
// thread's outputs, and adds back c (h[0] + sum of the taps that output o
// sums):
//   out[o] = h[0] (x[o] - c) + c D[o] + sum_j h[o-j] (x[j] - c),
//   D[o] = h[0] + sum_{j of the other parity} h[o-j]
//        = C - P(o+1) - Q(n-o),
// C = h[0] + the sum of every odd tap the filter reaches (offsets up to
// n-1 either way; it nearly cancels: formed in FP64 from the caller's taps),
// P(a) and Q(b) the sums of the odd taps at offsets >= a and <= -b (tails of
// small same-signed taps: FP32 suffix sums of the staged taps).  One extra
// warp forms C, P and Q while the others start their sums.
// Partial sums then stay near the size of the result (on a 2304 x 1472 fan
// sinogram: 1.3e-5 -> ~1e-6 from FP64).
#include "ctr_common.cuh"

namespace ctr {
namespace {

constexpr int kWeightChannels = 128;  // channels per CTA
constexpr int kWeightThreads = 256;
constexpr int kWeightRows = 32;       // rows per CTA
constexpr int kWeightPer = kWeightRows * kWeightChannels / kWeightThreads;  // elements per thread

// A CTA weights a block of kWeightRows x kWeightChannels: the FP64 weights of
// its channels are computed once into shared memory, then every thread loads
// all of its elements before storing any (correct in place: each element is
// read and written by one thread), so the loads are in flight together.
template <typename T>
__global__ void __launch_bounds__(kWeightThreads)
    fan_weight_kernel(const T* in, T* out, unsigned ns, unsigned long long rows, double ds,
                      double cents, double dso, double dsd, int type)
{
    __shared__ double s_w[kWeightChannels];
    const unsigned c0 = blockIdx.x * kWeightChannels;
    if (threadIdx.x < kWeightChannels) {
        const unsigned is = c0 + threadIdx.x;
        const double s = ds * (static_cast<double>(is) - cents);
        s_w[threadIdx.x] = type == 2 ? dso * fabs(cos(atan2(s, dsd))) / dsd : dso * fabs(cos(s / dsd)) / dsd;
    }
    __syncthreads();
    // launched as a dependent: the weights (kernel arguments only) are formed
    // while the kernel before it drains; global memory only after this wait
    grid_dep_wait();
    const unsigned long long r0 = static_cast<unsigned long long>(blockIdx.y) * kWeightRows;
    T v[kWeightPer];
#pragma unroll
    for (int i = 0; i < kWeightPer; ++i) {
        const int e = threadIdx.x + kWeightThreads * i;
        const unsigned long long r = r0 + e / kWeightChannels;
        const unsigned is = c0 + (e % kWeightChannels);
        v[i] = r < rows && is < ns ? in[r * ns + is] : T(0);
    }
#pragma unroll
    for (int i = 0; i < kWeightPer; ++i) {
        const int e = threadIdx.x + kWeightThreads * i;
        const unsigned long long r = r0 + e / kWeightChannels;
        const unsigned is = c0 + (e % kWeightChannels);
        if (r < rows && is < ns) out[r * ns + is] = static_cast<T>(s_w[e % kWeightChannels] * static_cast<double>(v[i]));
    }
}

template <typename T>
int launch_fan_weighting(const ctr_fan_weighting_param* p, const T* in, T* out, int batch,
                         cudaStream_t stream)
{
    if (!p || bad_ptr(in) || bad_ptr(out)) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->type != 1 && p->type != 2)
        return fail(CTR_ERR_INVALID_ARG, "fan weighting type %d (1 fan, 2 flat)", p->type);
    if (p->ns < 1 || p->nrow < 1) return fail(CTR_ERR_INVALID_ARG, "empty sinogram");
    const unsigned long long rows = static_cast<unsigned long long>(p->nrow) * batch;
    const double cents = static_cast<double>(p->ns - 1) / 2 + p->offset;
    dim3 grid(div_up(p->ns, kWeightChannels), div_up(rows, kWeightRows));
    if (grid.y > 65535u) return fail(CTR_ERR_UNSUPPORTED, "too many rows for one launch");
    const cudaError_t e = launch_dependent(fan_weight_kernel<T>, grid, dim3(kWeightThreads), 0, stream, in, out,
                                           p->ns, rows, p->ds, cents, p->dso, p->dsd, p->type);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "fan_weighting: %s", cudaGetErrorString(e));
    return check_launch("fan_weighting");
}

// ---- ramp filter ---------------------------------------------------------
//
// out[r][o] = ds * sum_j h[o - j] * x[r][j]   (correlation, the grad: h[j - o]).
// The ramp taps are zero at even offsets except 0, so output o sums the inputs
// of the other parity.  A thread computes 4 outputs of one parity, o_m = i0 + 2m,
// for kRows rows: stepping j by 2, the taps it needs, H[o_m - j], slide by one
// place (H[o_m - j - 2] = H[o_{m-1} - j]), so each step loads one new tap and
// one input per row for 4 * kRows FMAs, all from shared memory.  Thread pairs
// cover 8 consecutive outputs (both parities).  Even taps other than 0, which
// the ramp filters of the reference never have, take the generic loop.
constexpr int kFilterMaxThreads = 1024;
// Threads of the output tasks (the FP32 kernels add one warp, see filter_block).
constexpr int kFilterTaskThreads = kFilterMaxThreads - 32;
constexpr int kFilterPad = 16;   // zero taps beyond the ends of H
constexpr int kFilterRowsPlain = 2;
constexpr int kFilterRowsSpread = 3;

// Thread tasks of a row: (8-output block, parity).  When twice that fits one
// CTA, each task's inputs are split in two halves run by two threads, whose
// partial sums are added in a fixed order (halves the serial loop per thread).
__host__ __device__ inline int filter_tasks(unsigned ns) { return static_cast<int>((ns + 7) / 8) * 2; }
__host__ __device__ inline bool filter_split(unsigned ns) { return 2 * filter_tasks(ns) <= kFilterTaskThreads; }

__host__ __device__ inline int filter_threads(unsigned ns)
{
    const int t = filter_tasks(ns) * (filter_split(ns) ? 2 : 1);
    return t < 32 ? 32 : (t > kFilterTaskThreads ? kFilterTaskThreads : (t + 31) / 32 * 32);
}

// Tap storage: tap idx (offset d + ns - 1 + kFilterPad) lives at word
// tg*(idx/8) + idx%8.  With tg = 34 (skewed) a warp's lanes, which read taps
// i0 - j - 2 with i0 = 8q + p (q < 16, p < 2), fall in 32 distinct banks for
// every j; packed (tg = 8) the 16 groups of 8 fall in 8 banks (4-way
// conflicts).  The skewed layout is used where it fits the shared memory.
constexpr int kTapSkewed = 34, kTapPacked = 8;
__host__ __device__ inline int tap_slot(int idx, int tg) { return tg * (idx >> 3) + (idx & 7); }
__host__ __device__ inline int tap_words(unsigned ns, int tg)
{
    return tap_slot(2 * static_cast<int>(ns) + 2 * kFilterPad, tg);
}

// Shared layout (FP32): the tail sums P and Q of the odd taps [2][ns/2 + 2]
// and C (see filter_rows), then the taps H[-(ns-1) - kFilterPad .. ns - 1 +
// kFilterPad] (taps * ds), then xs[kRows][ns], then the second halves' sums
// [kRows][tasks][4].  FP64 has no tail sums.
__host__ __device__ inline size_t filter_tail_bytes(unsigned ns) { return (2 * (ns / 2 + 2) + 4) * sizeof(float); }
template <typename T>
__host__ __device__ inline size_t filter_smem(unsigned ns, int rows, int tg)
{
    return (sizeof(T) == 4 ? filter_tail_bytes(ns) : 0) +
           sizeof(T) * (static_cast<size_t>(tap_words(ns, tg)) + static_cast<size_t>(rows) * ns +
                        static_cast<size_t>(rows) * filter_tasks(ns) * 4);
}
// The FP32 kernels run one more warp, which forms C and the tail sums.
template <typename T>
__host__ __device__ inline int filter_block(unsigned ns)
{
    return filter_threads(ns) + (sizeof(T) == 4 ? 32 : 0);
}

// The tap layout for a launch: skewed when it fits kFilterSmemMax.
constexpr size_t kFilterSmemMax = 200 * 1024;
template <typename T>
inline int filter_layout(unsigned ns, int rows)
{
    return filter_smem<T>(ns, rows, kTapSkewed) <= kFilterSmemMax ? kTapSkewed : kTapPacked;
}

__device__ __forceinline__ float fma_t(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return fma(a, b, c); }

// Inputs j = j0, j0 + 2, ... < j1 (one parity) into the four outputs i0, i0 + 2,
// i0 + 4, i0 + 6 of kRows rows; w0..w3 are the taps of input j0.  (Blocked
// partial sums cut the FP32 rounding of the long sums by ~1.3x on phantom
// sinograms and cost 11 % of the filter's time; not kept.)
template <typename T, int kRows>
__device__ __forceinline__ void filter_span(const T* __restrict__ xs, int n, int j0, int j1, int i0, int tg,
                                            const T* __restrict__ H0, T w0, T w1, T w2, T w3,
                                            const T (&cr)[kRows], T (&acc)[kRows][4])
{
    const int d0 = (n - 1) + kFilterPad;  // tap d sits at H0[tap_slot(d + d0, tg)]
#pragma unroll 4
    for (int j = j0; j < j1; j += 2) {
#pragma unroll
        for (int r = 0; r < kRows; ++r) {
            const T xv = xs[r * n + j] - cr[r];
            acc[r][0] += w0 * xv;
            acc[r][1] += w1 * xv;
            acc[r][2] += w2 * xv;
            acc[r][3] += w3 * xv;
        }
        w3 = w2;
        w2 = w1;
        w1 = w0;
        w0 = H0[tap_slot(i0 - j - 2 + d0, tg)];
    }
}

template <typename T, int kRows, bool kGrad>
__device__ __forceinline__ void filter_rows(const T* __restrict__ in, const double* __restrict__ filter,
                                            T* __restrict__ out, const float* __restrict__ weight,
                                            unsigned ns, unsigned long long r0, int nr, double ds,
                                            int tg, unsigned char* smem_raw)
{
    constexpr bool kCentred = sizeof(T) == 4;
    const int n = static_cast<int>(ns);
    // FP32: the tail sums P [ns/2 + 2], Q [ns/2 + 2], then C
    const int nodd = n / 2;  // odd offsets in [1, n-1]
    float* Pt = reinterpret_cast<float*>(smem_raw);
    float* Qt = Pt + nodd + 2;
    float* Cs = Qt + nodd + 2;
    T* H0 = reinterpret_cast<T*>(smem_raw + (kCentred ? filter_tail_bytes(ns) : 0));
    const int d0 = (n - 1) + kFilterPad;  // tap d sits at H0[tap_slot(d + d0, tg)]
    auto H = [&](int d) -> T { return H0[tap_slot(d + d0, tg)]; };
    T* xs = H0 + tap_words(ns, tg);
    __shared__ int s_even;
    // the task threads; an FP32 block has one more warp (C and the tail sums)
    const int nthr = kCentred ? static_cast<int>(blockDim.x) - 32 : static_cast<int>(blockDim.x);

    const double* h = filter + ns;  // h[k], k in [-ns, ns]
    if (threadIdx.x == 0) s_even = 0;
    __syncthreads();
    {
        bool even = false;
        // staging loops unrolled so that a thread's global loads are in flight together
#pragma unroll 4
        for (int idx = threadIdx.x; idx < 2 * n + 2 * kFilterPad; idx += blockDim.x) {
            const int d = idx - (n - 1) - kFilterPad;
            double v = 0.0;
            if (d > -n && d < n) v = kGrad ? h[-d] : h[d];
            H0[tap_slot(idx, tg)] = static_cast<T>(v * ds);
            if (d != 0 && (d & 1) == 0 && v != 0.0) even = true;
        }
        if (even) s_even = 1;
#pragma unroll 4
        for (int idx = threadIdx.x; idx < kRows * n; idx += blockDim.x) {
            const int r = idx / n, j = idx - r * n;
            T v = 0;
            if (r < nr) {
                v = in[(r0 + r) * ns + j];
                if (weight) v = static_cast<T>(v * static_cast<T>(weight[j]));
            }
            xs[idx] = v;
        }
    }
    __syncthreads();
    if (kCentred && static_cast<int>(threadIdx.x) >= nthr) {
        // the extra warp, while the task threads start their sums.  Lanes 0-15
        // form P (positive offsets), lanes 16-31 Q (negative offsets): entry i
        // is the sum of the staged taps at odd offsets +-(2i+1) .. +-(n-1),
        // added from the far (small) end; entry nodd is 0.
        const int lane = threadIdx.x & 31, sl = lane & 15;
        const int sg = lane < 16 ? 1 : -1;
        float* A = lane < 16 ? Pt : Qt;
        const int C16 = (nodd + 15) / 16;
        const int i0 = min(sl * C16, nodd), i1 = min(i0 + C16, nodd);
        float tot = 0.0f;
        for (int i = i1 - 1; i >= i0; --i) tot += H(sg * (2 * i + 1));
        float suf = tot;  // inclusive suffix over this half's lanes
#pragma unroll
        for (int off = 1; off < 16; off <<= 1) {
            const float v = __shfl_down_sync(0xffffffffu, suf, off, 16);
            if (sl + off < 16) suf += v;
        }
        suf -= tot;
        for (int i = i1 - 1; i >= i0; --i) {
            suf += H(sg * (2 * i + 1));
            A[i] = suf;
        }
        if (sl == 0) A[nodd] = A[nodd + 1] = 0.0f;
        // C in FP64 from the caller's taps
        double cs = 0.0;
        for (int i = lane; i < nodd; i += 32) {
            const int k = 2 * i + 1;
            cs += kGrad ? h[-k] + h[k] : h[k] + h[-k];
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) cs += __shfl_xor_sync(0xffffffffu, cs, off);
        if (lane == 0) Cs[0] = static_cast<float>((h[0] + cs) * ds);
    }
    // the single-thread-per-task path writes outputs as it goes: it needs the
    // sums first
    if (kCentred && !filter_split(ns)) __syncthreads();
    // D[o] (FP32 kernels), once per output
    auto dcorr = [&](int o) -> T {
        if constexpr (kCentred) return Cs[0] - Pt[(o + 1) / 2] - Qt[(n - o) / 2];
        else return T(0);
    };
    // output o of a thread whose reference value is c (FP32: centred sums)
    auto finish = [&](int o, int r, T c, T D, T acc) -> T {
        if constexpr (kCentred) return fma_t(H(0), xs[r * n + o] - c, fma_t(c, D, acc));
        else return fma_t(H(0), xs[r * n + o], acc);
    };
    // reference value of a task's rows: the input next to its outputs
    auto refs = [&](int i0, T (&cr)[kRows]) {
#pragma unroll
        for (int r = 0; r < kRows; ++r) cr[r] = kCentred ? xs[r * n + min(i0 + 3, n - 1)] : T(0);
    };
    const int groups = filter_tasks(ns);  // thread tasks: (8-output block, parity)
    T* red = xs + kRows * n;              // [kRows][groups][4]
    if (!s_even && filter_split(ns)) {
        // two threads per task (nthr >= 2 * groups): inputs [jb, jm) and [jm, n)
        const int task = threadIdx.x;
        const bool active = task < 2 * groups;
        const int half = task >= groups ? 1 : 0;
        const int g = task - half * groups;
        const int i0 = (g >> 1) * 8 + (g & 1);
        T acc[kRows][4], cr[kRows];
#pragma unroll
        for (int r = 0; r < kRows; ++r)
#pragma unroll
            for (int m = 0; m < 4; ++m) acc[r][m] = 0;
        if (active) {
            refs(i0, cr);
            const int jb = (i0 + 1) & 1;  // inputs of the other parity
            const int jm = jb + 2 * ((n - jb + 1) / 4);
            const int j0 = half ? jm : jb, j1 = half ? n : jm;
            T w0 = H(i0 - j0), w1 = H(i0 + 2 - j0), w2 = H(i0 + 4 - j0), w3 = H(i0 + 6 - j0);
            filter_span<T, kRows>(xs, n, j0, j1, i0, tg, H0, w0, w1, w2, w3, cr, acc);
            if (half) {
#pragma unroll
                for (int r = 0; r < kRows; ++r)
#pragma unroll
                    for (int m = 0; m < 4; ++m) red[(r * groups + g) * 4 + m] = acc[r][m];
            }
        }
        __syncthreads();
        if (active && !half) {
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int o = i0 + 2 * m;
                if (o >= n) continue;
                const T D = dcorr(o);
#pragma unroll
                for (int r = 0; r < kRows; ++r)
                    if (r < nr)
                        out[(r0 + r) * ns + o] = finish(o, r, cr[r], D, acc[r][m] + red[(r * groups + g) * 4 + m]);
            }
        }
    } else if (!s_even) {
        for (int task = threadIdx.x; task < groups; task += blockDim.x) {
            const int i0 = (task >> 1) * 8 + (task & 1);
            T acc[kRows][4], cr[kRows];
#pragma unroll
            for (int r = 0; r < kRows; ++r)
#pragma unroll
                for (int m = 0; m < 4; ++m) acc[r][m] = 0;
            refs(i0, cr);
            const int jb = (i0 + 1) & 1;  // inputs of the other parity
            T w0 = H(i0 - jb), w1 = H(i0 + 2 - jb), w2 = H(i0 + 4 - jb), w3 = H(i0 + 6 - jb);
            filter_span<T, kRows>(xs, n, jb, n, i0, tg, H0, w0, w1, w2, w3, cr, acc);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int o = i0 + 2 * m;
                if (o >= n) continue;
                const T D = dcorr(o);
#pragma unroll
                for (int r = 0; r < kRows; ++r)
                    if (r < nr) out[(r0 + r) * ns + o] = finish(o, r, cr[r], D, acc[r][m]);
            }
        }
    } else {
        // a filter with even taps: the plain sum over every input
        for (int o = threadIdx.x; o < n; o += blockDim.x) {
            T acc[kRows];
#pragma unroll
            for (int r = 0; r < kRows; ++r) acc[r] = 0;
            for (int j = 0; j < n; ++j) {
                const T t = H(o - j);
#pragma unroll
                for (int r = 0; r < kRows; ++r) acc[r] += t * xs[r * n + j];
            }
#pragma unroll
            for (int r = 0; r < kRows; ++r)
                if (r < nr) out[(r0 + r) * ns + o] = acc[r];
        }
    }
    __syncthreads();  // shared buffers are free for the caller's next call
}

// kRows rows a CTA; with `spread` the rows are instead dealt evenly over the
// grid (CTA i: rows [i*rows/G, (i+1)*rows/G), at most kRows), so a grid of
// exactly the resident CTAs finishes in one wave.
template <typename T, bool kGrad, int kRows>
__global__ void __launch_bounds__(kFilterMaxThreads)
    ramp_filter_kernel(const T* __restrict__ in, const double* __restrict__ filter,
                       T* __restrict__ out, const float* __restrict__ weight, unsigned ns,
                       unsigned long long rows, double ds, int tg, int spread)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    grid_dep_wait();  // launched as a dependent of the kernel before it
    unsigned long long r0, r1;
    if (spread) {
        r0 = static_cast<unsigned long long>(blockIdx.x) * rows / gridDim.x;
        r1 = static_cast<unsigned long long>(blockIdx.x + 1) * rows / gridDim.x;
    } else {
        r0 = static_cast<unsigned long long>(blockIdx.x) * kRows;
        r1 = rows - r0 < kRows ? rows : r0 + kRows;
    }
    filter_rows<T, kRows, kGrad>(in, filter, out, weight, ns, r0, static_cast<int>(r1 - r0), ds, tg, smem_raw);
}

// Batched FP32 filtering with pre-weighting: one CTA per (job, row block).
__global__ void __launch_bounds__(kFilterMaxThreads)
    ramp_filter_batch_kernel(const FilterJob* __restrict__ jobs, const int2* __restrict__ blocks, int tg)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int2 b = blocks[blockIdx.x];  // (job, first row)
    const FilterJob J = jobs[b.x];
    const int nr = min(kFilterRowsPerBlock, static_cast<int>(J.nrow) - b.y);
    filter_rows<float, kFilterRowsPerBlock, false>(J.in, J.taps, J.out, J.weight, J.ns, b.y, nr,
                                                   J.ds, tg, smem_raw);
}

template <typename T, bool kGrad>
int launch_ramp_filter(const ctr_filter_param* p, const T* in, const double* filter, T* out,
                       const float* weight, int batch, cudaStream_t stream)
{
    if (!p || bad_ptr(in) || bad_ptr(filter) || bad_ptr(out))
        return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    if (p->ns < 1 || p->nrow < 1) return fail(CTR_ERR_INVALID_ARG, "empty sinogram");
    if (in == out) return fail(CTR_ERR_INVALID_ARG, "ramp filter cannot run in place");
    const unsigned long long rows = static_cast<unsigned long long>(p->nrow) * batch;
    const int threads = filter_block<T>(p->ns);
    // Up to kFilterRowsSpread rows a CTA dealt over the resident CTAs (one
    // wave, CTAs within a row of each other); more rows take CTAs of
    // kFilterRowsPlain rows in waves.
    {
        const int tg = filter_layout<T>(p->ns, kFilterRowsSpread);
        const size_t smem = filter_smem<T>(p->ns, kFilterRowsSpread, tg);
        auto kern = ramp_filter_kernel<T, kGrad, kFilterRowsSpread>;
        int per_sm = 0;
        if (smem <= kFilterSmemMax &&
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) ==
                cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) == cudaSuccess &&
            per_sm > 0) {
            const unsigned long long resident = static_cast<unsigned long long>(per_sm) * device_sms();
            if (rows <= kFilterRowsSpread * resident) {
                const unsigned blocks = static_cast<unsigned>(rows < resident ? rows : resident);
                const cudaError_t e = launch_dependent(kern, dim3(blocks), dim3(threads), smem, stream, in, filter,
                                                       out, weight, p->ns, rows, p->ds, tg, 1);
                if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "ramp_filter: %s", cudaGetErrorString(e));
                return check_launch("ramp_filter");
            }
        }
        cudaGetLastError();
    }
    const int tg = filter_layout<T>(p->ns, kFilterRowsPlain);
    const size_t smem = filter_smem<T>(p->ns, kFilterRowsPlain, tg);
    if (smem > kFilterSmemMax)
        return fail(CTR_ERR_UNSUPPORTED, "ns=%u exceeds the filter's shared-memory tile", p->ns);
    auto kern = ramp_filter_kernel<T, kGrad, kFilterRowsPlain>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "filter smem: %s", cudaGetErrorString(e));
    const unsigned blocks = div_up(rows, kFilterRowsPlain);
    e = launch_dependent(kern, dim3(blocks), dim3(threads), smem, stream, in, filter, out, weight, p->ns, rows,
                         p->ds, tg, 0);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "ramp_filter: %s", cudaGetErrorString(e));
    return check_launch("ramp_filter");
}

}  // namespace

int ramp_filter_weighted_f32(const ctr_filter_param* p, const float* in, const double* filter,
                             float* out, const float* weight, int batch, cudaStream_t stream)
{
    return launch_ramp_filter<float, false>(p, in, filter, out, weight, batch, stream);
}

// Batched weighting + filtering of a job list (see FilterJob); `blocks` lists
// (job, first row) pairs, one CTA each; max_ns sizes the shared memory.
int ramp_filter_batch_f32(const FilterJob* jobs, const int2* blocks, int n_blocks, unsigned max_ns,
                          cudaStream_t stream)
{
    const int tg = filter_layout<float>(max_ns, kFilterRowsPerBlock);
    const size_t smem = filter_smem<float>(max_ns, kFilterRowsPerBlock, tg);
    if (smem > kFilterSmemMax) return fail(CTR_ERR_UNSUPPORTED, "ns=%u too wide for the filter tile", max_ns);
    cudaError_t e = cudaFuncSetAttribute(ramp_filter_batch_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "filter smem: %s", cudaGetErrorString(e));
    if (n_blocks > 0)
        ramp_filter_batch_kernel<<<n_blocks, filter_block<float>(max_ns), smem, stream>>>(jobs, blocks, tg);
    return check_launch("ramp_filter_batch");
}

}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_fan_weighting_f32(const ctr_fan_weighting_param* p, const float* in, float* out,
                          int batch, cudaStream_t stream)
{
    return launch_fan_weighting<float>(p, in, out, batch, stream);
}
int ctr_fan_weighting_f64(const ctr_fan_weighting_param* p, const double* in, double* out,
                          int batch, cudaStream_t stream)
{
    return launch_fan_weighting<double>(p, in, out, batch, stream);
}
// The reference's grad applies the same diagonal weight (src/fan_weighting.cc:40-59).
int ctr_fan_weighting_grad_f32(const ctr_fan_weighting_param* p, const float* in, float* out,
                               int batch, cudaStream_t stream)
{
    return launch_fan_weighting<float>(p, in, out, batch, stream);
}
int ctr_fan_weighting_grad_f64(const ctr_fan_weighting_param* p, const double* in,
                               double* out, int batch, cudaStream_t stream)
{
    return launch_fan_weighting<double>(p, in, out, batch, stream);
}

int ctr_ramp_filter_f32(const ctr_filter_param* p, const float* in, const double* filter,
                        float* out, int batch, cudaStream_t stream)
{
    return launch_ramp_filter<float, false>(p, in, filter, out, nullptr, batch, stream);
}
int ctr_ramp_filter_f64(const ctr_filter_param* p, const double* in, const double* filter,
                        double* out, int batch, cudaStream_t stream)
{
    return launch_ramp_filter<double, false>(p, in, filter, out, nullptr, batch, stream);
}
int ctr_ramp_filter_grad_f32(const ctr_filter_param* p, const float* in, const double* filter,
                             float* out, int batch, cudaStream_t stream)
{
    return launch_ramp_filter<float, true>(p, in, filter, out, nullptr, batch, stream);
}
int ctr_ramp_filter_grad_f64(const ctr_filter_param* p, const double* in,
                             const double* filter, double* out, int batch,
                             cudaStream_t stream)
{
    return launch_ramp_filter<double, true>(p, in, filter, out, nullptr, batch, stream);
}

}  // extern "C"

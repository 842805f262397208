// Ramp filter on the BF16 tensor cores (tcgen05), for sinograms stored in
// FP32, BF16 or FP16.
//
// The ramp filter of src/filter.cc:67-91 (out[r][i] = ds * sum_j in[r][j] h[i-j],
// a zero-padded linear convolution; the grad, src/filter.cc:96-124, uses
// h[j-i]) is a product with the Toeplitz matrix T[i][j] = ds*h[i-j]:
// OUT = X T^T with M = rows (views x batch) and N = K = ns.  Both operands are
// split into BF16 terms, each the BF16 rounding of what the previous terms
// leave (the remainders are exact in FP32 for X and in FP64 for T):
//   2 terms (hi, lo; 16 significant bits):  OUT = X0 T0 + X0 T1 + X1 T0,
//   3 terms (hi, mid, lo; 24 bits):         OUT = X0 T0 + X0 T1 + X1 T0
//                                                + X0 T2 + X2 T0 + X1 T1,
// (products written X_a T_b^T), accumulating in FP32 in tensor memory.  The
// ramp taps sum to zero, so on a smooth sinogram the filter cancels almost
// all of its input and amplifies operand error about a hundredfold: with 2
// terms the filtered sinogram of a smooth 1472-channel fan sinogram is off by
// ~6e-4 (relative L2), with 3 terms by ~1e-6, below FP32 taps (~4e-6).
//
// Operand layout in HBM: each operand is stored already tiled the way the
// tensor core's shared-memory descriptor reads it.  A tile is 128 rows x 64 K
// elements, K-major with the 128-byte swizzle: row r of the tile starts at
// byte (r/8)*1024 + (r%8)*128, and its 16-byte chunk c is stored at chunk
// c ^ (r%8).  The term tiles of one (row tile, K block) follow each other (a
// block of 2 or 3 x 16 KiB); row tiles are outer and K blocks inner.  A
// pipeline stage of the GEMM is then two contiguous bulk copies (the X block
// and the T block), with no tensor map.  split_rows writes
// the X blocks and fuses the input conversion with the optional fan weighting
// (src/fan_weighting.cc:19-38).  split_toeplitz builds the T blocks once per
// plan from the FP64 taps.
//
// GEMM: one CTA per 128 x 128 output tile, 4 warps.  Thread 0 streams the K
// blocks into a ring of 192 KiB (3 stages of 64 KiB with 2 terms, 2 of 96 KiB
// with 3; full / empty mbarriers).  Thread 32 issues
// tcgen05.mma (M=128, N=128, K=16, BF16 x BF16 -> FP32) into a 128-column
// TMEM accumulator and frees each stage with tcgen05.commit.  After the last
// commit the four warps read their 32 TMEM lanes (tcgen05.ld 32x32b), stage
// the rows through shared memory and store them coalesced.  Every wait is
// bounded (about 1 s).  On a timeout the CTA raises kFlagWaitTimeout, waits
// for its copies in flight, frees its TMEM and returns without storing.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <vector>

#include "ctr_async.cuh"
#include "ctr_common.cuh"

struct ctr_ramp_tc_plan {
    int device;
    unsigned ns, nrow;
    int max_batch;
    int splits;             // BF16 terms per operand: 2 (hi, lo) or 3 (hi, mid, lo)
    unsigned kblocks;       // K blocks of 64 channels
    unsigned ntiles;        // output column tiles of 128 channels
    unsigned max_mtiles;    // row tiles of the X workspace
    unsigned char* T;       // split Toeplitz blocks, ntiles x kblocks x splits x 16 KiB
    unsigned char* X;       // split input blocks, max_mtiles x kblocks x splits x 16 KiB
    float* weight;          // per-channel fan weight, or null
};

namespace ctr {
namespace {

constexpr int kTcRows = 128;                         // rows of an operand tile (M or N)
constexpr int kTcK = 64;                             // K elements of a tile: 128 bytes of BF16
constexpr unsigned kTcTile = kTcRows * kTcK * 2;     // 16 KiB
constexpr unsigned kTcRing = 192 * 1024;             // pipeline ring
constexpr unsigned kTcSmem = kTcRing + 1024;         // + 1 KiB to align the ring

template <int kSplits>
struct TcShape {
    static constexpr unsigned kBlock = kSplits * kTcTile;   // the term tiles of one K block
    static constexpr unsigned kStage = 2 * kBlock;          // X block + T block
    static constexpr int kStages = static_cast<int>(kTcRing / kStage);
    static_assert(kStages >= 2, "ring too small");
};
constexpr unsigned kTcCols = 128;                    // TMEM columns of the FP32 accumulator
constexpr int kTcThreads = 128;
constexpr int kSplitThreads = 256;

// Byte offset of (row r, 16-byte chunk c) inside a 128-byte-swizzled tile.
__host__ __device__ __forceinline__ unsigned sw128_offset(unsigned r, unsigned c)
{
    return (r >> 3) * 1024u + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4);
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float to_f32(__half v) { return __half2float(v); }

// BF16 terms of two FP32 values, packed in pairs: term t is the BF16
// rounding of what terms 0..t-1 leave; every remainder is exact in FP32.
template <int kSplits>
__device__ __forceinline__ void split_pair(float a, float b, unsigned (&t)[kSplits])
{
#pragma unroll
    for (int i = 0; i < kSplits; ++i) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        const float2 hf = __bfloat1622float2(h);
        t[i] = *reinterpret_cast<const unsigned*>(&h);
        a -= hf.x;
        b -= hf.y;
    }
}

// One thread per 16-byte chunk (8 channels of one row) of the X blocks:
// converts, weights and splits, writing the chunk of every term tile.
// Rows past `rows` and channels past ns are zero.
template <typename Tin, int kSplits>
__global__ void __launch_bounds__(kSplitThreads)
    split_rows(const Tin* __restrict__ in, const float* __restrict__ weight,
               unsigned char* __restrict__ X, unsigned ns, unsigned long long rows,
               unsigned kblocks, unsigned long long nchunks)
{
    const unsigned long long g = static_cast<unsigned long long>(blockIdx.x) * kSplitThreads + threadIdx.x;
    if (g >= nchunks) return;
    const unsigned long long tile = g >> 10;  // 1024 chunks per tile
    const unsigned r = static_cast<unsigned>(g >> 3) & 127u, c = static_cast<unsigned>(g) & 7u;
    const unsigned long long rt = tile / kblocks;
    const unsigned kb = static_cast<unsigned>(tile - rt * kblocks);
    const unsigned long long row = rt * kTcRows + r;
    const unsigned k0 = kb * kTcK + c * 8;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const unsigned k = k0 + e;
        float x = 0.0f;
        if (row < rows && k < ns) {
            x = to_f32(in[row * ns + k]);
            if (weight) x *= __ldg(weight + k);
        }
        v[e] = x;
    }
    unsigned w[4][kSplits];
#pragma unroll
    for (int q = 0; q < 4; ++q) split_pair<kSplits>(v[2 * q], v[2 * q + 1], w[q]);
    unsigned char* dst = X + tile * TcShape<kSplits>::kBlock + sw128_offset(r, c);
#pragma unroll
    for (int i = 0; i < kSplits; ++i)
        *reinterpret_cast<uint4*>(dst + i * kTcTile) = make_uint4(w[0][i], w[1][i], w[2][i], w[3][i]);
}

// The T blocks: T[n][k] = ds*h[n-k] (grad: ds*h[k-n]) for n, k < ns, split in
// FP64 (every remainder exact), zero elsewhere.
template <int kSplits>
__global__ void __launch_bounds__(kSplitThreads)
    split_toeplitz(const double* __restrict__ taps, unsigned char* __restrict__ T, unsigned ns,
                   double ds, int grad, unsigned kblocks, unsigned long long nchunks)
{
    const unsigned long long g = static_cast<unsigned long long>(blockIdx.x) * kSplitThreads + threadIdx.x;
    if (g >= nchunks) return;
    const unsigned long long tile = g >> 10;
    const unsigned r = static_cast<unsigned>(g >> 3) & 127u, c = static_cast<unsigned>(g) & 7u;
    const unsigned long long nt = tile / kblocks;
    const unsigned kb = static_cast<unsigned>(tile - nt * kblocks);
    const long long n = static_cast<long long>(nt * kTcRows + r);
    const unsigned k0 = kb * kTcK + c * 8;
    unsigned short hs[kSplits][8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const long long k = k0 + e;
        double t = 0.0;
        if (n < ns && k < ns) t = ds * taps[static_cast<long long>(ns) + (grad ? k - n : n - k)];
#pragma unroll
        for (int i = 0; i < kSplits; ++i) {
            const __nv_bfloat16 h = __double2bfloat16(t);
            hs[i][e] = *reinterpret_cast<const unsigned short*>(&h);
            t -= static_cast<double>(__bfloat162float(h));
        }
    }
    unsigned char* dst = T + tile * TcShape<kSplits>::kBlock + sw128_offset(r, c);
#pragma unroll
    for (int i = 0; i < kSplits; ++i)
        *reinterpret_cast<uint4*>(dst + i * kTcTile) =
            make_uint4(hs[i][0] | (static_cast<unsigned>(hs[i][1]) << 16),
                       hs[i][2] | (static_cast<unsigned>(hs[i][3]) << 16),
                       hs[i][4] | (static_cast<unsigned>(hs[i][5]) << 16),
                       hs[i][6] | (static_cast<unsigned>(hs[i][7]) << 16));
}

// ---- tcgen05 pieces ------------------------------------------------------------

// Shared-memory matrix descriptor of a K-major, 128-byte-swizzled operand
// slice: start address >> 4 (bits 0-13), leading byte offset (bits 16-29,
// unused for swizzled K-major operands), stride between 8-row groups = 1024 B
// (bits 32-45, >> 4), descriptor version 1 (bits 46-47), base offset 0 (the
// tiles are 1024-byte aligned), swizzle mode 2 = 128 B (bits 61-63).  The
// K = 16 slice k of a tile starts 32*k bytes into it.
__device__ __forceinline__ unsigned long long sw128_desc(unsigned addr)
{
    return static_cast<unsigned long long>((addr & 0x3FFFFu) >> 4) | (1ull << 16) |
           (static_cast<unsigned long long>(1024u >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A
// and B BF16 (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) |
                              ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(unsigned tmem, unsigned long long a, unsigned long long b,
                                       unsigned accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(kTcIdesc), "r"(accumulate)
        : "memory");
}

// Arrives on `bar` once every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void tc_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Reads 32 consecutive FP32 columns of this warp's 32 TMEM lanes (lane i of
// the warp gets TMEM lane base + i); the load and its wait are one asm block,
// so no use of the registers can be scheduled before the data is there.
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32])
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// OUT[rows][ns] (FP32) = X T^T over the split blocks; grid (ntiles, mtiles).
template <int kSplits>
__global__ void __launch_bounds__(kTcThreads, 1)
    ramp_tc_gemm(const unsigned char* __restrict__ X, const unsigned char* __restrict__ T,
                 float* __restrict__ out, unsigned ns, unsigned long long rows, unsigned kblocks)
{
    constexpr int kTcStages = TcShape<kSplits>::kStages;
    constexpr unsigned kTcBlock = TcShape<kSplits>::kBlock, kTcStage = TcShape<kSplits>::kStage;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long s_full[kTcStages], s_empty[kTcStages], s_done;
    __shared__ unsigned s_tmem, s_issued, s_consumed;
    __shared__ int s_abort;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned raw = smem_u32(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;
    if (threadIdx.x == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(smem_u32(&s_full[s]), 1);
            mbar_init(smem_u32(&s_empty[s]), 1);
        }
        mbar_init(smem_u32(&s_done), 1);
        s_abort = 0;
        s_issued = 0;
        s_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&s_tmem)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = s_tmem;

    const unsigned char* Xb = X + static_cast<size_t>(blockIdx.y) * kblocks * kTcBlock;
    const unsigned char* Tb = T + static_cast<size_t>(blockIdx.x) * kblocks * kTcBlock;
    if (threadIdx.x == 0) {
        // producer: K block kb goes to stage kb % 3 once the MMAs of kb - 3 are done
        unsigned kb = 0;
        for (; kb < kblocks; ++kb) {
            const unsigned s = kb % kTcStages, u = kb / kTcStages;
            if (u > 0 && !mbar_wait_bounded(smem_u32(&s_empty[s]), (u - 1) & 1)) break;
            const unsigned full = smem_u32(&s_full[s]);
            mbar_expect_tx(full, kTcStage);
            bulk_load(base + s * kTcStage, Xb + static_cast<size_t>(kb) * kTcBlock, kTcBlock, full);
            bulk_load(base + s * kTcStage + kTcBlock, Tb + static_cast<size_t>(kb) * kTcBlock, kTcBlock,
                      full);
        }
        s_issued = kb;
        if (kb < kblocks) s_abort = 1;
    } else if (threadIdx.x == 32) {
        // MMA issuer: 4 K-slices x (3 or 6) term products per K block, the
        // products of term indices (a, b) with a + b < kSplits, plus (1, 1) for 3 terms
        unsigned kb = 0;
        for (; kb < kblocks; ++kb) {
            const unsigned s = kb % kTcStages, u = kb / kTcStages;
            if (!mbar_wait_bounded(smem_u32(&s_full[s]), u & 1)) break;
            tc_fence_after();
            const unsigned a = base + s * kTcStage, b = a + kTcBlock;
#pragma unroll
            for (int k = 0; k < kTcK / 16; ++k) {
                unsigned long long ad[kSplits], bd[kSplits];
#pragma unroll
                for (int i = 0; i < kSplits; ++i) {
                    ad[i] = sw128_desc(a + i * kTcTile + 32u * k);
                    bd[i] = sw128_desc(b + i * kTcTile + 32u * k);
                }
                tc_mma(tmem, ad[0], bd[0], (kb | k) != 0);
                tc_mma(tmem, ad[0], bd[1], 1u);
                tc_mma(tmem, ad[1], bd[0], 1u);
                if constexpr (kSplits == 3) {
                    tc_mma(tmem, ad[0], bd[2], 1u);
                    tc_mma(tmem, ad[2], bd[0], 1u);
                    tc_mma(tmem, ad[1], bd[1], 1u);
                }
            }
            tc_commit(smem_u32(&s_empty[s]));
        }
        s_consumed = kb;
        if (kb < kblocks) s_abort = 1;
        tc_commit(smem_u32(&s_done));  // arrives once every MMA above has completed
    }
    __syncwarp();
    const bool done = mbar_wait_bounded(smem_u32(&s_done), 0);
    tc_fence_after();
    if (!done) s_abort = 1;
    __syncthreads();

    if (s_abort) {
        if (threadIdx.x == 0) {
            raise_flag(kFlagWaitTimeout);
            // copies issued but never consumed must land before the CTA exits
            for (unsigned kb = s_consumed; kb < s_issued; ++kb)
                mbar_wait_bounded(smem_u32(&s_full[kb % kTcStages]), (kb / kTcStages) & 1);
        }
    } else {
        // epilogue: warp w owns TMEM lanes (tile rows) 32w..32w+31; each
        // 32 x 32 block goes through a padded shared tile (the ring is idle now)
        float* stage = reinterpret_cast<float*>(smem_raw + (base - raw)) + warp * 32 * 33;
        const unsigned long long row0 = static_cast<unsigned long long>(blockIdx.y) * kTcRows + warp * 32;
        const unsigned n0 = blockIdx.x * kTcRows;
#pragma unroll 1
        for (int cb = 0; cb < kTcRows / 32; ++cb) {
            float v[32];
            tmem_ld32(tmem + (static_cast<unsigned>(warp * 32) << 16) + cb * 32u, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) stage[lane * 33 + j] = v[j];
            __syncwarp();
            const unsigned n = n0 + cb * 32 + lane;
#pragma unroll 4
            for (int rr = 0; rr < 32; ++rr) {
                const unsigned long long row = row0 + rr;
                if (row < rows && n < ns) out[row * ns + n] = stage[rr * 33 + lane];
            }
            __syncwarp();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols)
                     : "memory");
    }
}

// FP64 fan weight of channel is (reference src/fan_weighting.cc:19-38).
double fan_weight(const ctr_fan_weighting_param& w, unsigned is)
{
    const double cents = static_cast<double>(w.ns - 1) / 2 + w.offset;
    const double s = w.ds * (static_cast<double>(is) - cents);
    return w.type == 2 ? w.dso * std::fabs(std::cos(std::atan2(s, w.dsd))) / w.dsd
                       : w.dso * std::fabs(std::cos(s / w.dsd)) / w.dsd;
}

unsigned long long split_chunks(unsigned tiles, unsigned kblocks)
{
    return static_cast<unsigned long long>(tiles) * kblocks * 1024ull;
}

unsigned block_bytes(int splits) { return splits * kTcTile; }

template <int kSplits>
int set_gemm_smem()
{
    cudaError_t e = cudaFuncSetAttribute(ramp_tc_gemm<kSplits>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(kTcSmem));
    return e == cudaSuccess ? CTR_OK : fail(CTR_ERR_CUDA, "tensor-core filter smem: %s", cudaGetErrorString(e));
}

template <int kSplits>
int run_splits(ctr_ramp_tc_plan* P, int in_dtype, const void* in, float* out, unsigned long long rows,
               cudaStream_t stream)
{
    const unsigned mtiles = div_up(rows, kTcRows);
    const unsigned long long nch = split_chunks(mtiles, P->kblocks);
    const unsigned sb = div_up(nch, kSplitThreads);
    switch (in_dtype) {
    case CTR_DTYPE_F32:
        split_rows<float, kSplits><<<sb, kSplitThreads, 0, stream>>>(static_cast<const float*>(in), P->weight,
                                                                     P->X, P->ns, rows, P->kblocks, nch);
        break;
    case CTR_DTYPE_BF16:
        split_rows<__nv_bfloat16, kSplits><<<sb, kSplitThreads, 0, stream>>>(
            static_cast<const __nv_bfloat16*>(in), P->weight, P->X, P->ns, rows, P->kblocks, nch);
        break;
    case CTR_DTYPE_F16:
        split_rows<__half, kSplits><<<sb, kSplitThreads, 0, stream>>>(static_cast<const __half*>(in), P->weight,
                                                                      P->X, P->ns, rows, P->kblocks, nch);
        break;
    default:
        return fail(CTR_ERR_INVALID_ARG, "input dtype %d (0 f32, 1 bf16, 2 f16)", in_dtype);
    }
    int st = check_launch("split_rows");
    if (st) return st;
    ramp_tc_gemm<kSplits><<<dim3(P->ntiles, mtiles), kTcThreads, kTcSmem, stream>>>(P->X, P->T, out, P->ns,
                                                                                    rows, P->kblocks);
    return check_launch("ramp_tc_gemm");
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_ramp_filter_tc_create(const ctr_filter_param* p, const double* filter,
                              const ctr_fan_weighting_param* weighting, int grad, int splits,
                              int max_batch, ctr_ramp_tc_plan** plan, cudaStream_t stream)
{
    if (!p || bad_ptr(filter) || !plan) return fail(CTR_ERR_INVALID_ARG, "null argument");
    *plan = nullptr;
    int st = check_common(max_batch);
    if (st) return st;
    if (p->ns < 1 || p->nrow < 1) return fail(CTR_ERR_INVALID_ARG, "empty sinogram");
    if (p->ns > 16384) return fail(CTR_ERR_UNSUPPORTED, "ns=%u above the tensor-core filter's 16384", p->ns);
    if (splits != 2 && splits != 3)
        return fail(CTR_ERR_INVALID_ARG, "splits %d (2: hi/lo, 3: hi/mid/lo)", splits);
    if (weighting) {
        if (weighting->type != 1 && weighting->type != 2)
            return fail(CTR_ERR_INVALID_ARG, "fan weighting type %d (1 fan, 2 flat)", weighting->type);
        if (weighting->ns != p->ns) return fail(CTR_ERR_INVALID_ARG, "weighting ns %u != filter ns %u",
                                                weighting->ns, p->ns);
    }
    const unsigned long long max_rows = static_cast<unsigned long long>(p->nrow) * max_batch;
    if (div_up(max_rows, kTcRows) > 65535u) return fail(CTR_ERR_UNSUPPORTED, "too many rows for one plan");
    st = splits == 2 ? set_gemm_smem<2>() : set_gemm_smem<3>();
    if (st) return st;
    auto* P = new ctr_ramp_tc_plan{};
    cudaGetDevice(&P->device);
    P->ns = p->ns;
    P->nrow = p->nrow;
    P->max_batch = max_batch;
    P->splits = splits;
    P->kblocks = div_up(p->ns, kTcK);
    P->ntiles = div_up(p->ns, kTcRows);
    P->max_mtiles = div_up(max_rows, kTcRows);
    const size_t tb = static_cast<size_t>(P->ntiles) * P->kblocks * block_bytes(splits);
    const size_t xb = static_cast<size_t>(P->max_mtiles) * P->kblocks * block_bytes(splits);
    cudaError_t e = cudaMalloc(&P->T, tb);
    if (e == cudaSuccess) e = cudaMalloc(&P->X, xb);
    if (e == cudaSuccess && weighting) {
        std::vector<float> w(p->ns);
        for (unsigned is = 0; is < p->ns; ++is) w[is] = static_cast<float>(fan_weight(*weighting, is));
        e = cudaMalloc(&P->weight, sizeof(float) * p->ns);
        if (e == cudaSuccess)
            e = cudaMemcpy(P->weight, w.data(), sizeof(float) * p->ns, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        ctr_ramp_filter_tc_destroy(P);
        return fail(CTR_ERR_CUDA, "tensor-core filter plan: %s", cudaGetErrorString(e));
    }
    const unsigned long long nch = split_chunks(P->ntiles, P->kblocks);
    const unsigned nb = div_up(nch, kSplitThreads);
    if (splits == 2)
        split_toeplitz<2><<<nb, kSplitThreads, 0, stream>>>(filter, P->T, p->ns, p->ds, grad != 0, P->kblocks, nch);
    else
        split_toeplitz<3><<<nb, kSplitThreads, 0, stream>>>(filter, P->T, p->ns, p->ds, grad != 0, P->kblocks, nch);
    st = check_launch("split_toeplitz");
    if (st) {
        ctr_ramp_filter_tc_destroy(P);
        return st;
    }
    *plan = P;
    return CTR_OK;
}

int ctr_ramp_filter_tc_run(ctr_ramp_tc_plan* P, int in_dtype, const void* in, float* out, int batch,
                           cudaStream_t stream)
{
    if (!P || bad_ptr(in) || bad_ptr(out)) return fail(CTR_ERR_INVALID_ARG, "null argument");
    int st = check_common(batch);
    if (st) return st;
    int dev = -1;
    cudaGetDevice(&dev);
    if (dev != P->device) return fail(CTR_ERR_INVALID_ARG, "plan made on device %d, current %d", P->device, dev);
    if (batch > P->max_batch) return fail(CTR_ERR_INVALID_ARG, "batch %d above the plan's %d", batch, P->max_batch);
    if (static_cast<const void*>(out) == in) return fail(CTR_ERR_INVALID_ARG, "ramp filter cannot run in place");
    const unsigned long long rows = static_cast<unsigned long long>(P->nrow) * batch;
    return P->splits == 2 ? run_splits<2>(P, in_dtype, in, out, rows, stream)
                          : run_splits<3>(P, in_dtype, in, out, rows, stream);
}

int ctr_ramp_filter_tc_info(const ctr_ramp_tc_plan* P, unsigned long long* workspace_bytes,
                            unsigned long long* mma_flops_per_row)
{
    if (!P) return fail(CTR_ERR_INVALID_ARG, "null plan");
    if (workspace_bytes)
        *workspace_bytes = (static_cast<unsigned long long>(P->ntiles) + P->max_mtiles) * P->kblocks *
                           block_bytes(P->splits);
    if (mma_flops_per_row)  // term products of 2 * (N tiles x 128) x (K blocks x 64) per row
        *mma_flops_per_row = (P->splits == 2 ? 3ull : 6ull) * 2ull * P->ntiles * kTcRows * P->kblocks * kTcK;
    return CTR_OK;
}

int ctr_ramp_filter_tc_destroy(ctr_ramp_tc_plan* P)
{
    if (!P) return CTR_OK;
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != P->device) cudaSetDevice(P->device);
    cudaFree(P->T);
    cudaFree(P->X);
    cudaFree(P->weight);
    if (cur != P->device && cur >= 0) cudaSetDevice(cur);
    delete P;
    return CTR_OK;
}

}  // extern "C"

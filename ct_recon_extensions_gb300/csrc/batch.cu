// Batched uneven fan-beam FBP: many sinograms, each with its own geometry
// (image size, views, channels), reconstructed by one batched weighting +
// ramp-filter launch and ONE persistent backprojection launch, the pair
// captured in a CUDA graph.
//
// The plan owns every per-item table (the reference's FP64 xpos/ypos/sincos,
// ramp taps, per-channel pre-weights), the filtered-sinogram workspace and the
// work list of (item, tile) pairs in longest-first order (cost = views x tile
// pixels).  Persistent CTAs (as many as are resident) take work items from an
// atomic counter, so items of very different sizes balance across the SMs.
// The tile body is the single-geometry FP32 backprojector's (bp_tile.cuh).
//
// Autotuning (CTR_PLAN_AUTOTUNE): the tile shape (32 x 64, 32 x 32 or 32 x 16 pixels)
// and the view-block depth (8 or 16 views per group) are chosen by timing each
// candidate on the plan's own batch once, at plan creation.
#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "bp_tile.cuh"
#include "host_geometry.h"

namespace ctr {
namespace {

struct ItemDev {
    TileConst c;
    const float* proj;  // filtered sinogram in the plan's workspace
    float* img;         // caller's output
    const double* xpos;
    const double* ypos;
    const double* sincos;
    int tiles_x;
};

// NG view groups of 256 threads per CTA.  8 rows per thread take up to 128
// registers: one 512-thread or two 256-thread CTAs per SM; fewer rows, twice that.
template <int R, int VB, int NG>
__global__ void __launch_bounds__(NG * kBpThreads, (R >= 8 ? 1 : 2) * (3 - NG))
    bp_fan_batch_f32(const ItemDev* __restrict__ items, const int2* __restrict__ work, int n_work,
                     int* __restrict__ counter)
{
    __shared__ int s_w;
    __shared__ __align__(16) TileConst s_c;  // the current item's constants
    constexpr int kWords = sizeof(TileConst) / sizeof(int);
    static_assert(sizeof(TileConst) % sizeof(int) == 0, "TileConst is copied word-wise");
    for (;;) {
        __syncthreads();  // every thread is done with the previous s_w and s_c
        if (threadIdx.x == 0) s_w = atomicAdd(counter, 1);
        __syncthreads();
        const int w = s_w;
        if (w >= n_work) return;
        const int2 wi = work[w];  // (item, tile)
        const ItemDev& it = items[wi.x];
        if (threadIdx.x < kWords)
            reinterpret_cast<int*>(&s_c)[threadIdx.x] = reinterpret_cast<const int*>(&it.c)[threadIdx.x];
        __syncthreads();
        const int tx = wi.y % it.tiles_x, ty = wi.y / it.tiles_x;
        if (!tile_forward<Geo::kFan, R, VB, NG>(it.proj, it.img, it.xpos, it.ypos, it.sincos, s_c, tx,
                                                ty, 0))
            return;
    }
}

struct Config {
    int R, VB, NG;
};
// Dynamic shared memory a candidate may take (227 KB per CTA, less static use).
constexpr size_t kBatchSmemMax = 220 * 1024;
constexpr Config kConfigs[] = {{4, 16, 2}, {2, 16, 2}, {4, 8, 2}, {2, 8, 2}, {8, 16, 2},
                               {8, 8, 2},  {8, 16, 1}, {8, 32, 1}};
constexpr int kNumConfigs = sizeof(kConfigs) / sizeof(kConfigs[0]);

template <int R, int VB, int NG>
void* batch_kernel()
{
    return reinterpret_cast<void*>(bp_fan_batch_f32<R, VB, NG>);
}

void* kernel_of(int ci)
{
    switch (ci) {
    case 0: return batch_kernel<4, 16, 2>();
    case 1: return batch_kernel<2, 16, 2>();
    case 2: return batch_kernel<4, 8, 2>();
    case 3: return batch_kernel<2, 8, 2>();
    case 4: return batch_kernel<8, 16, 2>();
    case 5: return batch_kernel<8, 8, 2>();
    case 6: return batch_kernel<8, 16, 1>();
    default: return batch_kernel<8, 32, 1>();
    }
}

template <typename T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    ~DevArray()
    {
        if (p) cudaFree(p);
    }
    bool alloc(size_t count)
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = count;
        return count == 0 || cudaMalloc(&p, count * sizeof(T)) == cudaSuccess;
    }
    bool upload(const std::vector<T>& v, cudaStream_t s)
    {
        if (!alloc(v.size())) return false;
        return v.empty() || cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                            s) == cudaSuccess;
    }
};

struct ConfigData {
    std::vector<ItemDev> h_items;
    DevArray<ItemDev> items;
    DevArray<int2> work;
    int n_work = 0;
    size_t smem = 0;
    int grid = 0;
};

}  // namespace
}  // namespace ctr

struct ctr_fbp_plan {
    int device = 0;
    int n = 0;
    int weighting = 1;
    std::vector<ctr_fan_bp_param> geoms;
    std::vector<std::unique_ptr<ctr::DevArray<double>>> xpos, ypos, sc, taps;
    std::vector<std::unique_ptr<ctr::DevArray<float>>> weights;
    ctr::DevArray<float> workspace;
    std::vector<ctr::FilterJob> h_jobs;
    ctr::DevArray<ctr::FilterJob> jobs;
    ctr::DevArray<int2> fblocks;
    int n_fblocks = 0;
    unsigned max_ns = 0;
    ctr::ConfigData cfg[ctr::kNumConfigs];
    int chosen = 6;  // without autotuning: 32 x 64 tiles, one group of 16 views, 2 CTAs per SM
    double tuned_ms = 0.0;
    bool autotuned = false;
    ctr::DevArray<int> counter;
    cudaStream_t stream = nullptr;  // creation / capture stream
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const float*> cur_proj;
    std::vector<float*> cur_img;
    unsigned long long workspace_bytes = 0;

    ~ctr_fbp_plan()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace ctr {
namespace {

TileConst item_const(const ctr_fan_bp_param& g, int tile_y, int R, int VB)
{
    TileConst c{};
    c.ns = g.ns; c.na = g.na; c.nx = g.nx; c.ny = g.ny;
    set_window(c, std::max(fan_window(g.ns, g.ds, g.dso, g.dsd, g.nx, g.ny, g.dx, g.dy, g.offset_x,
                                      g.offset_y, tile_y),
                           64 * R / VB));
    c.cents = static_cast<float>((g.ns - 1) / 2.0 + g.offset_s);
    c.nsm1 = static_cast<float>(g.ns - 1);
    c.dso = static_cast<float>(g.dso);
    c.K = static_cast<float>(g.dsd / g.ds);
    const double factor = std::round(std::fabs(g.na * g.orbit) / kPi);
    c.scale = static_cast<float>(g.dsd * g.dsd * std::fabs(g.orbit) / factor);
    c.ds_d = g.ds;
    c.cents_d = (g.ns - 1) / 2.0 + g.offset_s;
    c.dso_d = g.dso;
    c.dsd_d = g.dsd;
    c.dx = g.dx;
    c.dy = g.dy;
    c.dxf = static_cast<float>(g.dx);
    c.dyf = static_cast<float>(g.dy);
    fill_fan_tables(c, g.dsd, g.ds);
    c.proj_stride = static_cast<size_t>(g.ns) * g.na;
    c.img_stride = static_cast<size_t>(g.nx) * g.ny;
    c.total4 = static_cast<long long>(c.proj_stride & ~static_cast<size_t>(3));
    return c;
}

// Builds candidate ci; a candidate whose windows or shared memory do not fit
// is left out (n_work = 0), which is not an error unless every one is.
int build_config(ctr_fbp_plan* P, int ci, int sm_count)
{
    const int R = kConfigs[ci].R, VB = kConfigs[ci].VB, NG = kConfigs[ci].NG;
    const int ty = (kBpThreads / 32) * R, bv = NG * VB;
    ConfigData& D = P->cfg[ci];
    D.h_items.resize(P->n);
    std::vector<std::pair<double, int2>> work;
    size_t smem = 0;
    for (int i = 0; i < P->n; ++i) {
        const ctr_fan_bp_param& g = P->geoms[i];
        ItemDev& it = D.h_items[i];
        it.c = item_const(g, ty, R, VB);
        if (it.c.WB > 256) {
            D.n_work = 0;  // a window wider than the bulk-copy box
            return CTR_OK;
        }
        it.proj = P->h_jobs[i].out;
        it.img = nullptr;
        it.xpos = P->xpos[i]->p;
        it.ypos = P->ypos[i]->p;
        it.sincos = P->sc[i]->p;
        it.tiles_x = static_cast<int>(div_up(g.nx, kTileX));
        const int tiles_y = static_cast<int>(div_up(g.ny, ty));
        const double cost = static_cast<double>(g.na) * kTileX * ty;
        for (int t = 0; t < it.tiles_x * tiles_y; ++t) work.push_back({cost, make_int2(i, t)});
        smem = std::max(smem, 128 + 2 * static_cast<size_t>(bv) * it.c.WS * sizeof(float) +
                                  2 * static_cast<size_t>(bv) * it.c.W * sizeof(float2) +
                                  static_cast<size_t>(g.na) * kViewBytes);
    }
    // longest first; ties keep item order (tiles of one item stay together)
    std::stable_sort(work.begin(), work.end(),
                     [](const std::pair<double, int2>& a, const std::pair<double, int2>& b) {
                         return a.first > b.first;
                     });
    std::vector<int2> wl(work.size());
    for (size_t k = 0; k < work.size(); ++k) wl[k] = work[k].second;
    if (smem > kBatchSmemMax) {
        D.n_work = 0;
        return CTR_OK;
    }
    void* kern = kernel_of(ci);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "batch smem: %s", cudaGetErrorString(e));
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, NG * kBpThreads, smem);
    if (e != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        D.n_work = 0;
        return CTR_OK;
    }
    D.smem = smem;
    D.n_work = static_cast<int>(wl.size());
    D.grid = std::min(D.n_work, per_sm * sm_count);
    if (!D.work.upload(wl, P->stream) || !D.items.alloc(P->n))
        return fail(CTR_ERR_CUDA, "batch work list upload failed");
    return CTR_OK;
}

// Enqueue the whole batch (filter + backprojection) for config ci on stream s.
int enqueue(ctr_fbp_plan* P, int ci, cudaStream_t s)
{
    ConfigData& D = P->cfg[ci];
    int st = ramp_filter_batch_f32(P->jobs.p, P->fblocks.p, P->n_fblocks, P->max_ns, s);
    if (st) return st;
    cudaError_t e = cudaMemsetAsync(P->counter.p, 0, sizeof(int), s);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "counter reset: %s", cudaGetErrorString(e));
    void* args[] = {&D.items.p, &D.work.p, &D.n_work, &P->counter.p};
    e = cudaLaunchKernel(kernel_of(ci), dim3(D.grid), dim3(kConfigs[ci].NG * kBpThreads), args, D.smem, s);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
    return CTR_OK;
}

// Write the caller's pointers into the device descriptors of config ci.
int set_pointers(ctr_fbp_plan* P, int ci, const float* const* proj, float* const* img, cudaStream_t s)
{
    ConfigData& D = P->cfg[ci];
    for (int i = 0; i < P->n; ++i) {
        P->h_jobs[i].in = proj[i];
        D.h_items[i].img = img[i];
    }
    cudaError_t e = cudaMemcpyAsync(P->jobs.p, P->h_jobs.data(), P->n * sizeof(FilterJob),
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(D.items.p, D.h_items.data(), P->n * sizeof(ItemDev),
                            cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "descriptor update: %s", cudaGetErrorString(e));
    return CTR_OK;
}

int autotune(ctr_fbp_plan* P)
{
    // time each candidate on the batch itself: inputs = zeroed workspace-sized
    // sinograms, outputs = a scratch image set
    DevArray<float> in_all, out_all;
    size_t nin = 0, nout = 0;
    for (const auto& g : P->geoms) {
        nin += (static_cast<size_t>(g.ns) * g.na + 3) / 4 * 4;
        nout += static_cast<size_t>(g.nx) * g.ny;
    }
    if (!in_all.alloc(nin) || !out_all.alloc(nout)) return fail(CTR_ERR_CUDA, "autotune scratch");
    cudaMemsetAsync(in_all.p, 0, nin * sizeof(float), P->stream);
    std::vector<const float*> pin(P->n);
    std::vector<float*> pout(P->n);
    size_t oi = 0, oo = 0;
    for (int i = 0; i < P->n; ++i) {
        pin[i] = in_all.p + oi;
        pout[i] = out_all.p + oo;
        oi += (static_cast<size_t>(P->geoms[i].ns) * P->geoms[i].na + 3) / 4 * 4;
        oo += static_cast<size_t>(P->geoms[i].nx) * P->geoms[i].ny;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 1e30;
    int best_ci = 0;
    for (int ci = 0; ci < kNumConfigs; ++ci) {
        if (P->cfg[ci].n_work == 0) continue;
        int st = set_pointers(P, ci, pin.data(), pout.data(), P->stream);
        if (!st) st = enqueue(P, ci, P->stream);  // warm-up
        if (st) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return st;
        }
        cudaEventRecord(e0, P->stream);
        for (int rep = 0; rep < 2; ++rep) enqueue(P, ci, P->stream);
        cudaEventRecord(e1, P->stream);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / 2 < best) {
            best = ms / 2;
            best_ci = ci;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaStreamSynchronize(P->stream);
    if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    P->chosen = best_ci;
    P->tuned_ms = best;
    P->autotuned = true;
    return CTR_OK;
}

}  // namespace
}  // namespace ctr

using namespace ctr;

extern "C" {

int ctr_fbp_fan_plan_create(const ctr_fan_bp_param* geoms, int n_items, int weighting,
                            int flags, ctr_fbp_plan** out)
{
    if (!out) return fail(CTR_ERR_INVALID_ARG, "null plan pointer");
    *out = nullptr;
    if (!geoms || n_items < 1) return fail(CTR_ERR_INVALID_ARG, "need at least one item");
    if (weighting != 1 && weighting != 2)
        return fail(CTR_ERR_INVALID_ARG, "weighting %d (1 fan, 2 flat)", weighting);
    int st = ctr_device_check();
    if (st) return st;
    auto P = std::make_unique<ctr_fbp_plan>();
    cudaGetDevice(&P->device);
    int sm_count = 0;
    cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, P->device);
    if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(CTR_ERR_CUDA, "plan stream");
    P->n = n_items;
    P->weighting = weighting;
    P->geoms.assign(geoms, geoms + n_items);
    // per-item tables and the workspace
    size_t ws = 0;
    std::vector<size_t> off(n_items);
    for (int i = 0; i < n_items; ++i) {
        const ctr_fan_bp_param& g = P->geoms[i];
        if (g.ns < 1 || g.na < 1 || g.nx < 1 || g.ny < 1 || !(g.ds != 0.0) || !(g.dsd != 0.0))
            return fail(CTR_ERR_INVALID_ARG, "item %d: invalid geometry", i);
        if (g.na > 4096) return fail(CTR_ERR_UNSUPPORTED, "item %d: more than 4096 views", i);
        off[i] = ws;
        ws += (static_cast<size_t>(g.ns) * g.na + 3) / 4 * 4;  // 16-byte aligned items
        P->max_ns = std::max(P->max_ns, g.ns);
    }
    if (!P->workspace.alloc(ws)) return fail(CTR_ERR_CUDA, "workspace of %zu floats", ws);
    P->workspace_bytes = ws * sizeof(float);
    P->h_jobs.resize(n_items);
    std::vector<int2> blocks;
    for (int i = 0; i < n_items; ++i) {
        const ctr_fan_bp_param& g = P->geoms[i];
        std::vector<double> xp, yp, sc, taps, w;
        pixel_positions(g.nx, g.ny, g.dx, g.dy, g.offset_x, g.offset_y, xp, yp);
        fan_sincos(g.na, g.orbit_start, g.orbit, sc);
        ramp_taps(g.ns, g.ds, g.dsd, weighting == 1 ? 1 : 2, taps);
        fan_weights(g.ns, g.ds, g.offset_s, g.dso, g.dsd, weighting, w);
        std::vector<float> wf(w.begin(), w.end());
        P->xpos.emplace_back(new DevArray<double>());
        P->ypos.emplace_back(new DevArray<double>());
        P->sc.emplace_back(new DevArray<double>());
        P->taps.emplace_back(new DevArray<double>());
        P->weights.emplace_back(new DevArray<float>());
        if (!P->xpos[i]->upload(xp, P->stream) || !P->ypos[i]->upload(yp, P->stream) ||
            !P->sc[i]->upload(sc, P->stream) || !P->taps[i]->upload(taps, P->stream) ||
            !P->weights[i]->upload(wf, P->stream) || cudaStreamSynchronize(P->stream) != cudaSuccess)
            return fail(CTR_ERR_CUDA, "item %d: table upload failed", i);
        FilterJob& J = P->h_jobs[i];
        J.in = nullptr;
        J.out = P->workspace.p + off[i];
        J.taps = P->taps[i]->p;
        J.weight = P->weights[i]->p;
        J.ns = g.ns;
        J.nrow = g.na;
        J.ds = g.ds;
        for (unsigned r = 0; r < g.na; r += kFilterRowsPerBlock) blocks.push_back(make_int2(i, static_cast<int>(r)));
    }
    P->n_fblocks = static_cast<int>(blocks.size());
    if (!P->fblocks.upload(blocks, P->stream) || !P->jobs.alloc(n_items) || !P->counter.alloc(1))
        return fail(CTR_ERR_CUDA, "plan descriptors");
    for (int ci = 0; ci < kNumConfigs; ++ci) {
        st = build_config(P.get(), ci, sm_count);
        if (st) return st;
    }
    if (P->cfg[P->chosen].n_work == 0) {
        for (int ci = 0; ci < kNumConfigs; ++ci)
            if (P->cfg[ci].n_work > 0) {
                P->chosen = ci;
                break;
            }
        if (P->cfg[P->chosen].n_work == 0)
            return fail(CTR_ERR_UNSUPPORTED, "no backprojection tile shape fits these items' windows");
    }
    if (cudaStreamSynchronize(P->stream) != cudaSuccess) return fail(CTR_ERR_CUDA, "plan setup");
    if (flags & CTR_PLAN_AUTOTUNE) {
        st = autotune(P.get());
        if (st) return st;
    }
    // capture filter + persistent backprojection once; descriptors are read
    // from device memory, so the graph serves every later pointer set
    if (flags & CTR_PLAN_GRAPH) {
        if (cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return fail(CTR_ERR_CUDA, "graph capture");
        st = enqueue(P.get(), P->chosen, P->stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(P->stream, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess || cudaGraphInstantiate(&P->exec, g, 0) != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return fail(CTR_ERR_CUDA, "graph instantiate");
        }
        P->graph = g;
    }
    *out = P.release();
    return CTR_OK;
}

int ctr_fbp_fan_plan_run(ctr_fbp_plan* P, const float* const* proj, float* const* img,
                         cudaStream_t stream)
{
    if (!P || !proj || !img) return fail(CTR_ERR_INVALID_ARG, "null argument");
    for (int i = 0; i < P->n; ++i) {
        if (!proj[i] || !img[i]) return fail(CTR_ERR_INVALID_ARG, "item %d: null pointer", i);
        if (reinterpret_cast<uintptr_t>(proj[i]) % 4 != 0)
            return fail(CTR_ERR_INVALID_ARG, "item %d: misaligned sinogram", i);
    }
    const bool same = static_cast<int>(P->cur_proj.size()) == P->n &&
                      std::equal(proj, proj + P->n, P->cur_proj.begin()) &&
                      std::equal(img, img + P->n, P->cur_img.begin());
    if (!same) {
        const int st = set_pointers(P, P->chosen, proj, img, stream);
        if (st) return st;
        P->cur_proj.assign(proj, proj + P->n);
        P->cur_img.assign(img, img + P->n);
    }
    if (P->exec) {
        const cudaError_t e = cudaGraphLaunch(P->exec, stream);
        if (e != cudaSuccess) return fail(CTR_ERR_CUDA, "graph launch: %s", cudaGetErrorString(e));
        return CTR_OK;
    }
    return enqueue(P, P->chosen, stream);
}

int ctr_fbp_fan_plan_info(const ctr_fbp_plan* P, ctr_fbp_plan_info* info)
{
    if (!P || !info) return fail(CTR_ERR_INVALID_ARG, "null argument");
    const ConfigData& D = P->cfg[P->chosen];
    info->n_items = P->n;
    info->work_items = D.n_work;
    info->tile_rows = (kBpThreads / 32) * kConfigs[P->chosen].R;
    info->view_block = kConfigs[P->chosen].VB;
    info->ctas = D.grid;
    info->autotuned = P->autotuned ? 1 : 0;
    info->tuned_ms = P->tuned_ms;
    info->graph = P->exec != nullptr;
    info->workspace_bytes = P->workspace_bytes;
    long long kernels = 3;  // filter, counter reset, backprojection
    info->launches_per_run = kernels;
    return CTR_OK;
}

int ctr_fbp_fan_plan_destroy(ctr_fbp_plan* P)
{
    delete P;
    return CTR_OK;
}

}  // extern "C"

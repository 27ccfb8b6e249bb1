// fs_batch_api.cu -- C ABI of the ragged batch: many independent systems (different
// particle counts, slice counts, temperatures and walker counts) swept by one persistent
// kernel launch, optionally replayed from a CUDA graph.  No counterpart in the reference,
// which builds one OpenCL program per system (FeynSimul/kernel.py:53-457).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/feynsimul.h"

extern int fsi_thread_error(int code, const char *msg);
std::string fsi_float_literals(const std::string &s);
std::string fsi_prelude(bool dbl);
const char *fsi_rng_src();
const char *fsi_batch_src();
int fsi_nskip_for(int lux);
int fsi_compile(const std::string &src, bool fast, std::string *cubin, std::string *log);

#define FS_BATCH_MAX_S 10

struct FsBatchSysHost {  // mirrors FsBatchSys in fs_batch.cuh
    float *paths;
    float *old_scratch;
    float *vcache;
    uint32_t *seeds, *wseeds, *rtab, *gtab, *accepts;
    double *op_sums;
    int n_walkers, N, S, tpw, wpb, nops, type, n_tiles;
    int op_runs, msteps;
    int global;
    float eps;
    float sigma[FS_BATCH_MAX_S + 1];
};

struct fs_batch {
    int device = 0;
    std::vector<fs_batch_system> sys;
    std::vector<int> sys_global;  // per system: paths worked on in device memory
    std::vector<int> type_dof;
    std::vector<FsBatchSysHost> desc;
    int n_ops = 0, block = 256, grid = 0;
    int lux = -1;  // RANLUX luxuaryFactor as the user gives it (the kernel uses +1); -1: xorshift
    size_t smem = 0, old_slot = 0;
    long long n_items = 0, node_updates = 0;
    int regs = 0;
    std::string log, source;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kern = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    void *d_desc = nullptr, *d_items = nullptr, *d_counter = nullptr, *d_old = nullptr;
    std::vector<void *> allocs;
    bool timed = false;
};

static int bfail(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return fsi_thread_error(code, buf);
}

#define BT(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return bfail(FS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static size_t tile_smem_bytes(int dof, int N, int S, int wpb, int nops)
{
    long long dstride = N + (N >> S);
    long long wstride = (long long)dof * dstride;
    wstride = ((wstride + 15) / 16) * 16;
    if ((wstride / 16) % 2 == 0) wstride += 16;
    return (size_t)(wpb * wstride) * 4 + (size_t)wpb * std::max(nops, 1) * 8;
}

static void free_batch(fs_batch *b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : b->allocs) cudaFree(p);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->lib) cudaLibraryUnload(b->lib);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

static int balloc(fs_batch *b, void **p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(FS_ERR_OOM, "Unable to allocate global memory on device, out of memory? (%zu bytes)", bytes);
    }
    b->allocs.push_back(*p);
    BT(cudaMemsetAsync(*p, 0, bytes ? bytes : 16, b->stream));
    return FS_OK;
}

// RANLUX rows of a device table seeded by ranluxcl_init from xs (host), in slices of the
// no-alloc seeding's row limit, in the batch's stream
static int seed_rows(fs_batch *b, uint32_t *table, const uint64_t *xs, size_t n_rows)
{
    const size_t slice = 1u << 18;
    for (size_t r = 0; r < n_rows; r += slice) {
        const size_t n = std::min(slice, n_rows - r);
        int rc = fs_ranlux_init_noalloc(table + r * 28, xs + r, n, b->stream);
        if (rc) return rc;
        cudaError_t e = cudaStreamSynchronize(b->stream);  // the seeding's scratch is reused
        if (e != cudaSuccess) return bfail(FS_ERR_CUDA, "ranlux seeding: %s", cudaGetErrorString(e));
    }
    return FS_OK;
}

extern "C" int fs_batch_create(int32_t n_types, const int32_t *type_dof, const char *const *potentials,
                               const char *const *user_codes, const char *const *operators, int32_t n_ops,
                               int32_t n_systems, const fs_batch_system *systems, int32_t op_runs,
                               int32_t msteps, int32_t block_threads, int32_t ranlux_luxury, fs_batch **out)
{
    if (!out || n_types < 1 || n_systems < 1 || !type_dof || !potentials || !systems)
        return bfail(FS_ERR_CONFIG, "fs_batch_create: bad arguments");
    if (n_ops < 0 || n_ops > 4 || op_runs < 1 || msteps < 0)
        return bfail(FS_ERR_CONFIG, "fs_batch_create: 0..4 operators, op_runs >= 1, msteps >= 0");
    if (block_threads < 32 || block_threads > 1024 || block_threads % 32)
        return bfail(FS_ERR_CONFIG, "fs_batch_create: block_threads must be a multiple of 32 in [32, 1024]");
    if (ranlux_luxury != -1) {
        // the single-system rule (fs_create): luxury 0-3, or >= 23 with p - 24 a multiple of 4
        const int lux = ranlux_luxury + 1, ns = fsi_nskip_for(lux);
        if (ranlux_luxury < 0 || (lux > 4 && lux < 24) || ns % 4 != 0 || (ns != 0 && ns < 24))
            return bfail(FS_ERR_CONFIG, "fs_batch_create: ranlux_luxury must be -1 (xorshift), 0-3, or >= 23 "
                                        "with p - 24 a multiple of 4");
    }
    *out = nullptr;
    fs_batch *b = new fs_batch();
    b->block = block_threads;
    b->lux = ranlux_luxury;
    b->n_ops = n_ops;
    b->type_dof.assign(type_dof, type_dof + n_types);
    b->sys.assign(systems, systems + n_systems);
    size_t max_smem = 0, max_old = 0;
    for (int i = 0; i < n_systems; i++) {
        fs_batch_system &s = b->sys[i];
        if (s.type < 0 || s.type >= n_types) { free_batch(b); return bfail(FS_ERR_CONFIG, "system %d: bad type", i); }
        const int dof = b->type_dof[s.type];
        if (dof < 1 || dof > 64) { free_batch(b); return bfail(FS_ERR_CONFIG, "type %d: DOF must be 1..64", s.type); }
        if (s.n_slices < 2 || (s.n_slices & (s.n_slices - 1)) || s.bisection_level < 1 ||
            s.bisection_level > FS_BATCH_MAX_S || (1 << s.bisection_level) > s.n_slices || s.n_walkers < 1 ||
            !(s.beta > 0)) {
            free_batch(b);
            return bfail(FS_ERR_CONFIG, "system %d: N a power of 2, 1 <= S <= min(10, log2 N), walkers >= 1, beta > 0", i);
        }
        const int tpw = s.n_slices >> s.bisection_level;
        if (tpw > block_threads || (tpw > 32 && tpw % 32)) {
            free_batch(b);
            return bfail(FS_ERR_CONFIG, "system %d: N / 2^S = %d threads per walker does not fit the block", i, tpw);
        }
        int wpb_max = std::min(s.walkers_per_tile > 0 ? s.walkers_per_tile : block_threads, block_threads / tpw);
        if (tpw > 32) wpb_max = std::min(wpb_max, 15);  // named barriers 1..15
        int wpb = wpb_max;
        while (wpb > 1 && tile_smem_bytes(dof, s.n_slices, s.bisection_level, wpb, n_ops) > 200 * 1024) wpb--;
        // walkers so large that shared memory holds too few of them to fill half the CTA
        // (large clusters at N = 1024) work on their paths in device memory instead
        const bool global = wpb * tpw * 2 < block_threads && dof > 8;
        size_t tile_bytes;
        if (global) {
            wpb = wpb_max;
            tile_bytes = (size_t)wpb * std::max(n_ops, 1) * 8;
        } else {
            tile_bytes = tile_smem_bytes(dof, s.n_slices, s.bisection_level, wpb, n_ops);
            if (tile_bytes > 220 * 1024) {
                free_batch(b);
                return bfail(FS_ERR_CONFIG, "system %d: one walker's path does not fit in shared memory", i);
            }
        }
        b->sys_global.push_back(global ? 1 : 0);
        s.walkers_per_tile = wpb;
        max_smem = std::max(max_smem, tile_bytes);
        const size_t seg = (size_t)1 << s.bisection_level;
        // saved segment, and with the potential cache (3 or more DOF) its cached values
        max_old = std::max(max_old, (seg - 1) * (dof + (dof >= 3 ? 1 : 0)) * (size_t)(wpb * tpw));
        b->node_updates += (long long)s.n_walkers * tpw * (long long)(seg - 1) * op_runs * msteps;
    }
    b->smem = max_smem;
    b->old_slot = (max_old + 31) / 32 * 32;

    // ---- source: prelude, RNG, one namespace per type, batch kernel, dispatcher ----
    std::ostringstream o;
    o << fsi_prelude(false) << "#define FS_NSKIP " << (b->lux >= 0 ? fsi_nskip_for(b->lux + 1) : 0)
      << "\n#define FSB_RANLUX " << (b->lux >= 0 ? 1 : 0) << "\n" << fsi_rng_src() << "\n";
    for (int k = 0; k < n_types; k++) {
        const int dof = b->type_dof[k];
        // scalar-argument bodies; called rather than inlined for more than 8 DOF (see the
        // same rule in fs_api.cu): the dispatcher holds every type's sweep
        std::ostringstream args, call;
        for (int d = 0; d < dof; d++) {
            args << (d ? ", " : "") << "float x" << (d + 1);
            call << (d ? ", " : "") << "x[" << d << "]";
        }
        const char *inl = dof > 8 ? "__device__ __noinline__ " : "__device__ __forceinline__ ";
        o << "namespace fs_type_" << k << " {\n" << fsi_float_literals(user_codes && user_codes[k] ? user_codes[k] : "")
          << "\n" << inl << "float pot_s(" << args.str() << ") {\n        return ("
          << fsi_float_literals(potentials[k]) << ");\n}\n"
          << inl << "void ops_s(" << args.str() << ", float *o) {\n";
        for (int j = 0; j < n_ops; j++)
            o << "        o[" << j << "] = (" << fsi_float_literals(operators[k * n_ops + j]) << ");\n";
        if (n_ops == 0) o << "        (void)o;\n";
        o << "}\nstruct Sys {\n    static const int NOPS = " << n_ops << ";\n"
          << "    static __device__ __forceinline__ float pot(const float *x) { return pot_s(" << call.str()
          << "); }\n"
          << "    static __device__ __forceinline__ void ops(const float *x, float *o) { ops_s(" << call.str()
          << ", o); }\n};\n}\n";
    }
    o << fsi_batch_src() << "\n";
    // one register budget for every CTA size up to 512, so the autotuner's candidates share
    // one compiled module
    o << "extern \"C\" __global__ void __launch_bounds__(" << (block_threads <= 512 ? 512 : block_threads)
      << ") fs_batch_kernel(const FsBatchSys *sys, const FsBatchItem *items, int n_items, int *counter, "
         "unsigned long long old_slot)\n{\n"
         "    extern __shared__ __align__(16) float fsb_smem[];\n"
         "    __shared__ int s_it;\n"
         "    for (;;) {\n"
         "        if (threadIdx.x == 0) s_it = atomicAdd(counter, 1);\n"
         "        __syncthreads();\n"
         "        const int it = s_it;\n"
         "        __syncthreads();\n"
         "        if (it >= n_items) break;\n"
         "        const FsBatchItem item = items[it];\n"
         "        const FsBatchSys &sd = sys[item.sys];\n"
         "        switch (sd.type * 2 + sd.global) {\n";
    // one case per (type, path placement) pair the batch uses
    std::vector<char> used(2 * n_types, 0);
    for (int i = 0; i < n_systems; i++) used[2 * b->sys[i].type + b->sys_global[i]] = 1;
    for (int k = 0; k < n_types; k++)
        for (int g = 0; g < 2; g++)
            if (used[2 * k + g])
                o << "        case " << (2 * k + g) << ": fs_batch_tile<" << b->type_dof[k] << ", fs_type_" << k
                  << "::Sys, " << (g ? "true" : "false") << ">(sd, item.tile, fsb_smem, old_slot); break;\n";
    o << "        default: break;\n        }\n    }\n}\n";
    b->source = o.str();
    std::string cubin;
    int rc = fsi_compile(b->source, true, &cubin, &b->log);
    if (rc) {
        free_batch(b);
        return rc;
    }
    cudaError_t e = cudaGetDevice(&b->device);
    if (e != cudaSuccess) {
        free_batch(b);
        return bfail(FS_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
    }
#define CT(x)                   \
    do {                        \
        int r_ = (x);           \
        if (r_) {               \
            free_batch(b);      \
            return r_;          \
        }                       \
    } while (0)
    auto cuda = [&](cudaError_t err, const char *what) -> int {
        return err == cudaSuccess ? FS_OK : bfail(FS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
    };
    CT(cuda(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "cudaStreamCreate"));
    CT(cuda(cudaEventCreate(&b->ev0), "cudaEventCreate"));
    CT(cuda(cudaEventCreate(&b->ev1), "cudaEventCreate"));
    CT(cuda(cudaLibraryLoadData(&b->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0), "load"));
    CT(cuda(cudaLibraryGetKernel(&b->kern, b->lib, "fs_batch_kernel"), "fs_batch_kernel"));
    CT(cuda(cudaFuncSetAttribute((const void *)b->kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem),
            "smem attribute"));
    {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, (const void *)b->kern) == cudaSuccess) b->regs = fa.numRegs;
        else cudaGetLastError();
        int per_sm = 0, nsm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)b->kern, b->block, b->smem);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device);
        cudaGetLastError();
        b->grid = std::max(1, per_sm) * std::max(1, nsm);
    }

    // ---- buffers, descriptors, work items (largest tiles first) ----
    std::vector<std::pair<double, std::pair<int, int>>> items;
    b->desc.resize(n_systems);
    CT(balloc(b, &b->d_old, (size_t)b->grid * b->old_slot * 4));
    for (int i = 0; i < n_systems; i++) {
        const fs_batch_system &s = b->sys[i];
        FsBatchSysHost &d = b->desc[i];
        memset(&d, 0, sizeof d);
        const int dof = b->type_dof[s.type];
        d.n_walkers = s.n_walkers;
        d.N = s.n_slices;
        d.S = s.bisection_level;
        d.tpw = s.n_slices >> s.bisection_level;
        d.wpb = s.walkers_per_tile;
        d.nops = n_ops;
        d.type = s.type;
        d.n_tiles = (s.n_walkers + d.wpb - 1) / d.wpb;
        d.op_runs = op_runs;
        d.msteps = msteps;
        d.global = b->sys_global[i];
        // epsilon and the bisection widths in FP32 as the single-system kernel forms them
        char lit[64];
        snprintf(lit, sizeof lit, "%1.17e", s.beta / (double)s.n_slices);
        d.eps = strtof(lit, nullptr);
        const float seg = (float)(1 << d.S);
        for (int n = 0; n <= d.S; n++) {
            volatile float prod = seg * d.eps;
            volatile float q = prod / (2.0f * (float)(1 << n));
            d.sigma[n] = n == 0 ? (float)prod : std::sqrt((float)q);
        }
        const size_t W = s.n_walkers, T = W * d.tpw;
        void *p;
        CT(balloc(b, &p, W * dof * s.n_slices * 4)); d.paths = (float *)p;
        if (dof >= 3) {
            CT(balloc(b, &p, W * s.n_slices * 4)); d.vcache = (float *)p;  // potential cache
        }
        CT(balloc(b, &p, T * 16)); d.seeds = (uint32_t *)p;
        CT(balloc(b, &p, W * 16)); d.wseeds = (uint32_t *)p;
        if (b->lux >= 0) {
            // RANLUX tables, seeded with distinct default values per system and row (callers
            // re-seed with fs_batch_init_ranlux)
            CT(balloc(b, &p, T * 28 * 4)); d.rtab = (uint32_t *)p;
            CT(balloc(b, &p, W * 28 * 4)); d.gtab = (uint32_t *)p;
            std::vector<uint64_t> xs(std::max(T, W));
            for (size_t r = 0; r < T; r++) xs[r] = ((uint64_t)(0x5EED0000u + (unsigned)i) << 32) + r;
            CT(seed_rows(b, d.rtab, xs.data(), T));
            for (size_t r = 0; r < W; r++) xs[r] = ((uint64_t)(0x7EED0000u + (unsigned)i) << 32) + r;
            CT(seed_rows(b, d.gtab, xs.data(), W));
        }
        CT(balloc(b, &p, T * 4)); d.accepts = (uint32_t *)p;
        CT(balloc(b, &p, W * std::max(n_ops, 1) * 8)); d.op_sums = (double *)p;
        d.old_scratch = (float *)b->d_old;
        const double cost = (double)d.wpb * d.tpw * ((1 << d.S) - 1) * dof * (double)dof;
        for (int t = 0; t < d.n_tiles; t++) items.push_back({cost, {i, t}});
    }
    std::stable_sort(items.begin(), items.end(), [](const auto &a, const auto &c) { return a.first > c.first; });
    std::vector<int> flat;
    for (auto &it : items) {
        flat.push_back(it.second.first);
        flat.push_back(it.second.second);
    }
    b->n_items = (long long)items.size();
    CT(balloc(b, &b->d_desc, b->desc.size() * sizeof(FsBatchSysHost)));
    CT(balloc(b, &b->d_items, flat.size() * 4));
    CT(balloc(b, &b->d_counter, 16));
    CT(cuda(cudaMemcpyAsync(b->d_desc, b->desc.data(), b->desc.size() * sizeof(FsBatchSysHost),
                            cudaMemcpyHostToDevice, b->stream), "desc"));
    CT(cuda(cudaMemcpyAsync(b->d_items, flat.data(), flat.size() * 4, cudaMemcpyHostToDevice, b->stream), "items"));
    CT(cuda(cudaStreamSynchronize(b->stream), "sync"));
#undef CT
    *out = b;
    return FS_OK;
}

extern "C" int fs_batch_destroy(fs_batch *b)
{
    if (!b) return FS_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_batch(b);
    return FS_OK;
}

static int launch_once(fs_batch *b)
{
    BT(cudaMemsetAsync(b->d_counter, 0, 4, b->stream));
    int n_items = (int)b->n_items;
    unsigned long long old_slot = b->old_slot;
    void *args[] = {&b->d_desc, &b->d_items, &n_items, &b->d_counter, &old_slot};
    BT(cudaLaunchKernel((const void *)b->kern, dim3(b->grid), dim3(b->block), args, b->smem, b->stream));
    return FS_OK;
}

extern "C" int fs_batch_run(fs_batch *b, int32_t n_launches, int32_t use_graph)
{
    if (!b || n_launches < 1) return bfail(FS_ERR_CONFIG, "fs_batch_run: bad arguments");
    BT(cudaSetDevice(b->device));
    if (use_graph && !b->gexec) {
        // capture counter reset + persistent launch once; replay it per launch
        BT(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        int rc = launch_once(b);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc) return rc;
        if (e != cudaSuccess) return bfail(FS_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
        b->graph = g;
        BT(cudaGraphInstantiate(&b->gexec, g, 0));
    }
    BT(cudaEventRecord(b->ev0, b->stream));
    for (int i = 0; i < n_launches; i++) {
        if (use_graph) {
            BT(cudaGraphLaunch(b->gexec, b->stream));
        } else {
            int rc = launch_once(b);
            if (rc) return rc;
        }
    }
    BT(cudaEventRecord(b->ev1, b->stream));
    b->timed = true;
    return FS_OK;
}

extern "C" int fs_batch_sync(fs_batch *b)
{
    if (!b) return FS_ERR_CONFIG;
    BT(cudaStreamSynchronize(b->stream));
    return FS_OK;
}

extern "C" int fs_batch_get_run_time(fs_batch *b, double *seconds)
{
    if (!b || !seconds || !b->timed) return bfail(FS_ERR_STATE, "no batch run yet");
    BT(cudaEventSynchronize(b->ev1));
    float ms = 0.f;
    BT(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    *seconds = ms * 1e-3;
    return FS_OK;
}

static int sys_copy(fs_batch *b, int32_t i, void *dev, void *host, size_t bytes, size_t expect, bool in)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    if (bytes != expect) return bfail(FS_ERR_IO, "buffer has %zu bytes, expected %zu", bytes, expect);
    BT(cudaSetDevice(b->device));
    BT(cudaMemcpyAsync(in ? dev : host, in ? host : dev, bytes, in ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                       b->stream));
    BT(cudaStreamSynchronize(b->stream));
    return FS_OK;
}

extern "C" int fs_batch_set_paths(fs_batch *b, int32_t i, const float *host, size_t n)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    const fs_batch_system &s = b->sys[i];
    return sys_copy(b, i, b->desc[i].paths, (void *)host, n * 4,
                    (size_t)s.n_walkers * b->type_dof[s.type] * s.n_slices * 4, true);
}

extern "C" int fs_batch_get_paths(fs_batch *b, int32_t i, float *host, size_t n)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    const fs_batch_system &s = b->sys[i];
    return sys_copy(b, i, b->desc[i].paths, host, n * 4, (size_t)s.n_walkers * b->type_dof[s.type] * s.n_slices * 4,
                    false);
}

extern "C" int fs_batch_set_seeds(fs_batch *b, int32_t i, const uint32_t *thread_rows, size_t n_threads,
                                  const uint32_t *walker_rows, size_t n_walkers)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    const FsBatchSysHost &d = b->desc[i];
    int rc = sys_copy(b, i, d.seeds, (void *)thread_rows, n_threads * 16, (size_t)d.n_walkers * d.tpw * 16, true);
    if (!rc) rc = sys_copy(b, i, d.wseeds, (void *)walker_rows, n_walkers * 16, (size_t)d.n_walkers * 16, true);
    return rc;
}

extern "C" int fs_batch_init_ranlux(fs_batch *b, int32_t i, const uint64_t *xs_threads, size_t n_threads,
                                    const uint64_t *xs_walkers, size_t n_walkers)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    if (b->lux < 0) return bfail(FS_ERR_STATE, "the batch was created with xorshift streams");
    const FsBatchSysHost &d = b->desc[i];
    if (!xs_threads || !xs_walkers || n_threads != (size_t)d.n_walkers * d.tpw || n_walkers != (size_t)d.n_walkers)
        return bfail(FS_ERR_IO, "system %d: %d thread seeds and %d walker seeds expected", i, d.n_walkers * d.tpw,
                     d.n_walkers);
    BT(cudaSetDevice(b->device));
    int rc = seed_rows(b, d.rtab, xs_threads, n_threads);
    return rc ? rc : seed_rows(b, d.gtab, xs_walkers, n_walkers);
}

extern "C" int fs_batch_get_ranlux_tables(fs_batch *b, int32_t i, uint32_t *thread_rows, size_t n_threads,
                                          uint32_t *walker_rows, size_t n_walkers)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    if (b->lux < 0) return bfail(FS_ERR_STATE, "the batch was created with xorshift streams");
    const FsBatchSysHost &d = b->desc[i];
    int rc = sys_copy(b, i, d.rtab, thread_rows, n_threads * 28 * 4, (size_t)d.n_walkers * d.tpw * 28 * 4, false);
    return rc ? rc : sys_copy(b, i, d.gtab, walker_rows, n_walkers * 28 * 4, (size_t)d.n_walkers * 28 * 4, false);
}

extern "C" int fs_batch_get_op_sums(fs_batch *b, int32_t i, double *out, size_t n)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    const FsBatchSysHost &d = b->desc[i];
    return sys_copy(b, i, d.op_sums, out, n * 8, (size_t)d.n_walkers * std::max(b->n_ops, 1) * 8, false);
}

extern "C" int fs_batch_get_accepts(fs_batch *b, int32_t i, uint32_t *out, size_t n)
{
    if (!b || i < 0 || i >= (int)b->sys.size()) return bfail(FS_ERR_CONFIG, "bad system index");
    const FsBatchSysHost &d = b->desc[i];
    return sys_copy(b, i, d.accepts, out, n * 4, (size_t)d.n_walkers * d.tpw * 4, false);
}

extern "C" int fs_batch_query(const fs_batch *b, int64_t *node_updates_per_launch, int64_t *smem_bytes,
                              int64_t *registers, int64_t *n_items, int64_t *grid, int64_t *walkers_per_tile,
                              size_t n_systems)
{
    if (!b) return FS_ERR_CONFIG;
    if (node_updates_per_launch) *node_updates_per_launch = b->node_updates;
    if (smem_bytes) *smem_bytes = (int64_t)b->smem;
    if (registers) *registers = b->regs;
    if (n_items) *n_items = b->n_items;
    if (grid) *grid = b->grid;
    if (walkers_per_tile)
        for (size_t i = 0; i < n_systems && i < b->sys.size(); i++) walkers_per_tile[i] = b->sys[i].walkers_per_tile;
    return FS_OK;
}

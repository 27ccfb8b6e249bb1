// fs_api.cu -- host side of libfeynsimul_gb300.so: the C ABI declared in include/feynsimul.h.
//
// The reference builds one OpenCL program per run configuration from a text template
// (FeynSimul/kernel.py:215-381).  This library does the same for sm_103a: it validates the
// configuration (kernel.py:93-211), generates CUDA source (FS_* constants + the device RNG
// header + the plugin's userCode / potential / operators / correlators + fs_pimc.cuh),
// compiles it with NVRTC (cached per source text, in memory and on disk), loads it with
// cudaLibraryLoadData and owns every device buffer of the run.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <sys/stat.h>
#include <unistd.h>

#include "../../include/feynsimul.h"

static const char *kRngSrc =
#include "fs_rng.inc"
    ;
static const char *kPimcSrc =
#include "fs_pimc.inc"
    ;
static const char *kMlpSrc =
#include "fs_mlp.inc"
    ;
static const char *kBatchSrc =
#include "fs_batch.inc"
    ;
__attribute__((visibility("hidden"))) const char *fsi_batch_src() { return kBatchSrc; }

#define FS_VERSION "feynsimul_gb300 0.1 (sm_103a)"
// sizes of the learned-proposal model (fs_mlp.cuh: 16-128-128-128-16)
#define FS_MLP_FRAG_BYTES ((1 * 16 + 8 * 16 + 8 * 16 + 8 * 2) * 32 * 8)
#define FS_MLP_NBIAS_FLOATS (128 * 3 + 16)

// ------------------------------------------------------------------ errors
static thread_local std::string g_thread_err;

// host image of the device's precision-study correlator accumulator (fs_pimc.cuh FsCorAcc)
struct FsCorStudyHost {
    double d;
    float f, ks, kc, pad;
};
static_assert(sizeof(FsCorStudyHost) == 24, "study accumulator layout");

struct fs_handle {
    fs_config cfg{};
    int device = 0;
    std::string source, log, err;
    std::vector<std::string> ops, cors, hists;
    // launch geometry
    int tpw = 1, seg = 1, wpb = 1, block = 1, grid = 1;
    int cor_ilv = 0;  // correlator lags summed in one slice pass over a doubled slice buffer
    int pipe = 0;     // correlator helpers one measurement behind the movers (FS_PIPE)
    long long snstride = 0;  // FS_PIPE: one path snapshot in shared memory, elements
    int mx = 1;       // thread groups per CTA: 1 moving + mx - 1 summing correlator lags (FS_MX)
    long long cwstride = 0;  // per-walker correlator buffer in shared memory, elements
    int resident_per_sm = 0;  // resident CTAs per SM of the sweep kernel (fs_run_host), 0 = not yet queried
    long long wstride = 0, vstride = 0;
    int vglobal = 0;  // potential cache in device memory (FS_VGLOBAL) instead of shared memory
    long long n_threads = 0;
    size_t smem = 0;
    int regs = 0;
    size_t ft = 4, op_elem = 8, cor_elem = 8;
    size_t n_ops_elems = 0, n_cor_elems = 0, n_cor_lags = 0, n_bins = 0, n_hist = 0;
    double *d_red = nullptr;  // fs_reduce_correlator output (sum, sumsq)
    void *d_shift_old = nullptr;  // path shift, fixed mode: row saved before the move
    void *d_vcache = nullptr;     // potential cache in device memory: [walkers][N]
    unsigned long long steps_done = 0;  // Metropolis steps of all launches so far
    int last_chunks = 0;                // chunks (kernel launches per sweep set) of the last fs_run_host
    // CUDA objects
    cudaLibrary_t lib = nullptr;
    cudaKernel_t k_metro = nullptr, k_rinit = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t s_in = nullptr, s_out = nullptr;  // fs_run_host copy streams
    cudaStream_t s_comp2 = nullptr;                 // fs_run_host: second compute stream
    double *d_wops = nullptr;                       // fs_get_walker_operators output
    std::vector<cudaEvent_t> ev_chunk;               // fs_run_host: copy-in / compute done per chunk
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    // device buffers
    void *d_paths = nullptr;
    uint32_t *d_accepts = nullptr, *d_seeds = nullptr, *d_snap = nullptr, *d_wseeds = nullptr;
    uint32_t *d_rtab = nullptr, *d_gtab = nullptr, *d_bins = nullptr;
    void *d_ops = nullptr, *d_cor = nullptr;
    unsigned long long *d_hist = nullptr;
    int *d_status = nullptr;   // [0] FS_STATUS_* flags, [1] 1 + a walker that raised one
    bool status_pending = false;  // a sweep ran since fs_sync last read d_status
    void *d_mlp_frag = nullptr;
    float *d_mlp_bias = nullptr;
    double mlp_inv_scale = 1.0;
    size_t g_rows = 0;
    size_t device_bytes = 0;
};

static int fail(fs_handle *h, int code, const char *fmt, ...)
{
    char buf[2048];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h)
        h->err = buf;
    else
        g_thread_err = buf;
    return code;
}

// error reporting for the library's other translation units (not exported)
__attribute__((visibility("hidden"))) int fsi_thread_error(int code, const char *msg)
{
    return fail(nullptr, code, "%s", msg);
}

#define CUDA_TRY(h, call, code)                                                              \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail((h), (code), "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                        __FILE__, __LINE__);                                                 \
    } while (0)

// ------------------------------------------------------------------ code generation
// Append 'f' to unsuffixed floating literals: the reference compiles plugin code with
// -cl-single-precision-constant (kernel.py:376-377); CUDA would otherwise promote
// expressions such as 0.5*x to FP64.
static std::string float_literals(const std::string &s)
{
    std::string out;
    size_t i = 0, n = s.size();
    out.reserve(n + 16);
    auto dig = [&](size_t k) { return k < n && std::isdigit((unsigned char)s[k]); };
    while (i < n) {
        char c = s[i];
        if (c == '/' && i + 1 < n && s[i + 1] == '/') {
            size_t e = s.find('\n', i);
            e = e == std::string::npos ? n : e;
            out.append(s, i, e - i);
            i = e;
            continue;
        }
        if (c == '/' && i + 1 < n && s[i + 1] == '*') {
            size_t e = s.find("*/", i + 2);
            e = e == std::string::npos ? n : e + 2;
            out.append(s, i, e - i);
            i = e;
            continue;
        }
        if (c == '"' || c == '\'') {
            size_t e = i + 1;
            while (e < n && s[e] != c) e += (s[e] == '\\') ? 2 : 1;
            e = std::min(n, e + 1);
            out.append(s, i, e - i);
            i = e;
            continue;
        }
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t e = i;
            while (e < n && (std::isalnum((unsigned char)s[e]) || s[e] == '_')) e++;
            out.append(s, i, e - i);
            i = e;
            continue;
        }
        if (std::isdigit((unsigned char)c) || (c == '.' && dig(i + 1))) {
            size_t j = i;
            bool fl = false;
            if (c == '0' && j + 1 < n && (s[j + 1] == 'x' || s[j + 1] == 'X')) {
                j += 2;
                while (j < n && (std::isxdigit((unsigned char)s[j]) || s[j] == '.')) {
                    if (s[j] == '.') fl = true;
                    j++;
                }
                if (j < n && (s[j] == 'p' || s[j] == 'P')) {
                    fl = true;
                    j++;
                    if (j < n && (s[j] == '+' || s[j] == '-')) j++;
                    while (dig(j)) j++;
                }
            } else {
                while (dig(j)) j++;
                if (j < n && s[j] == '.') {
                    fl = true;
                    j++;
                    while (dig(j)) j++;
                }
                if (j < n && (s[j] == 'e' || s[j] == 'E')) {
                    size_t k = j + 1;
                    if (k < n && (s[k] == '+' || s[k] == '-')) k++;
                    if (dig(k)) {
                        fl = true;
                        j = k;
                        while (dig(j)) j++;
                    }
                }
            }
            size_t k = j;
            while (k < n && (std::isalpha((unsigned char)s[k]) || s[k] == '_')) k++;
            out.append(s, i, k - i);
            if (fl && k == j) out += 'f';
            i = k;
            continue;
        }
        out += c;
        i++;
    }
    return out;
}

static std::string fmt17(double v)
{
    char b[64];
    snprintf(b, sizeof b, "%1.17e", v);  // the reference's '%1.17e' (kernel.py:298, :312)
    return b;
}

static int nskip_for(int lux)
{
    switch (lux) {
    case 0: return 0;
    case 1: return 24;
    case 2: return 76;
    case 3: return 200;
    case 4: return 380;
    default: return lux - 24;
    }
}

// The bisection widths sigma_n = sqrt(2^S eps / 2^(n+1)) (kernel.c:608-618), evaluated with
// the same IEEE operations the reference's kernel performs in FLOAT_TYPE (eps rounded from
// its '%1.17e' literal), emitted as exact hexadecimal constants.
static std::string sigma_table(int S, double eps_d, bool dbl)
{
    std::ostringstream o;
    o << "__constant__ FT fs_sigma[" << (S + 1) << "] = {";
    const std::string lit = fmt17(eps_d);
    char b[64];
    if (dbl) {
        const double e = strtod(lit.c_str(), nullptr);
        const double seg = (double)(1 << S);
        for (int i = 0; i <= S; i++) {
            double v = i == 0 ? seg * e : std::sqrt(seg * e / (2.0 * (double)(1 << i)));
            snprintf(b, sizeof b, "%a", v);
            o << (i ? ", " : "") << b;
        }
    } else {
        const float e = strtof(lit.c_str(), nullptr);
        const float seg = (float)(1 << S);
        for (int i = 0; i <= S; i++) {
            volatile float prod = seg * e;
            volatile float den = 2.0f * (float)(1 << i);
            volatile float q = prod / den;
            float v = i == 0 ? (float)prod : std::sqrt((float)q);
            snprintf(b, sizeof b, "%a", (double)v);
            o << (i ? ", " : "") << b << "f";
        }
    }
    o << "};\n";
    return o.str();
}

static std::string gen_prelude(bool dbl)
{
    std::ostringstream o;
    o << "// generated by libfeynsimul_gb300 (" FS_VERSION ")\n";
    o << "#define FS_DOUBLE " << (dbl ? 1 : 0) << "\n";
    if (dbl) {
        o << "typedef double FT;\n#define M_PI 3.14159265358979323846\n#define M_PI_2 1.57079632679489661923\n";
    } else {
        o << "typedef float FT;\n#define M_PI 3.14159265358979323846f\n#define M_PI_2 1.57079632679489661923f\n";
    }
    o << "#define FLOAT_TYPE FT\n#define FLOAT_TYPE_VECTOR FT##4\n";
    // OpenCL built-in spellings accepted in plugin strings (physical_systems/__init__.py:5-9)
    o << "#define native_exp exp\n#define native_log log\n#define native_sqrt sqrt\n"
         "#define native_sin sin\n#define native_cos cos\n#define native_powr pow\n"
         "#define native_divide(a, b) ((a) / (b))\n#define native_recip(a) ((FT)1 / (a))\n"
         "#define half_exp exp\n#define half_log log\n#define half_sqrt sqrt\n";
    return o.str();
}

struct GenOut {
    std::string src;
};

static std::string gen_source(const fs_handle &h, const std::string &potential,
                              const std::string &user_code)
{
    const fs_config &c = h.cfg;
    const bool dbl = c.enable_double != 0;
    auto lit = [&](double v) { return fmt17(v) + (dbl ? "" : "f"); };
    auto cvt = [&](const std::string &s) { return dbl ? s : float_literals(s); };
    std::ostringstream o;
    o << gen_prelude(dbl);
    const int nhist = c.hist_bins > 0 ? (int)h.hists.size() : 0;
    const double opnorm = 1.0 / ((double)c.operator_runs * c.n_slices * c.n_walkers / (double)h.n_threads);
    o << "#define FS_DOF " << c.dof << "\n#define FS_N " << c.n_slices << "\n#define FS_S "
      << c.bisection_level << "\n#define FS_SEG " << h.seg << "\n#define FS_TPW " << h.tpw
      << "\n#define FS_WPB " << h.wpb << "\n#define FS_MINB " << c.min_blocks_per_sm
      << "\n#define FS_WSTRIDE " << h.wstride
      << "\n#define FS_NWALKERS " << c.n_walkers
      << "\n#define FS_WPG " << c.walkers_per_group << "\n#define FS_NWG "
      << (c.n_walkers / std::max(1, c.walkers_per_group)) << "\n#define FS_PARALLEL "
      << (c.enable_parallelize_path ? 1 : 0) << "\n#define FS_RANLUX " << (c.enable_ranlux ? 1 : 0)
      << "\n#define FS_NSKIP " << (c.enable_ranlux ? nskip_for(c.luxury_factor + 1) : 0)
      << "\n#define FS_COMPAT " << (c.compat ? 1 : 0) << "\n#define FS_ACCUM " << c.accum
      << "\n#define FS_PARTIALS " << c.partials
      << "\n#define FS_FAST " << (c.fast_math ? 1 : 0) << "\n#define FS_NOPS " << h.ops.size()
      << "\n#define FS_NCOR " << h.cors.size() << "\n#define FS_OPRUNS " << c.operator_runs
      << "\n#define FS_MSTEPS " << c.metro_steps_per_operator_run << "\n#define FS_EPS "
      << lit(c.beta / (double)c.n_slices) << "\n#define FS_OPNORM " << lit(opnorm)
      << "\n#define FS_BINS " << (c.enable_bins ? 1 : 0) << "\n#define FS_NHIST " << nhist
      << "\n#define FS_LEARNED " << (c.learned ? 1 : 0) << "\n#define FS_GLOBAL " << (c.global_path ? 1 : 0)
      << "\n#define FS_VCACHE " << (h.vstride || h.vglobal ? 1 : 0) << "\n#define FS_VSTRIDE " << h.vstride
      << "\n#define FS_VGLOBAL " << h.vglobal
      << "\n#define FS_COR_ILV " << h.cor_ilv << "\n#define FS_CWSTRIDE " << h.cwstride << "\n#define FS_MX "
      << h.mx << "\n#define FS_PIPE " << h.pipe << "\n#define FS_SNSTRIDE " << h.snstride << "\n";
    {
        const int mv = c.moves ? c.moves : FS_MOVE_BISECTION;
        const double nb = (double)c.n_slices / c.beta;
        o << "#define FS_BISECT " << ((mv & FS_MOVE_BISECTION) ? 1 : 0) << "\n#define FS_PATH_SHIFT "
          << ((mv & FS_MOVE_PATH_SHIFT) ? 1 : 0) << "\n#define FS_SNM " << ((mv & FS_MOVE_SINGLE_NODE) ? 1 : 0)
          << "\n#define FS_EPS_INV2 " << lit(nb * nb) << "\n#define FS_ALPHA " << lit(c.alpha)
          << "\n#define FS_PSALPHA " << lit(c.ps_alpha) << "\n";  // kernel.py:298-299, :326, :329
    }
    {
        char b[64];
        snprintf(b, sizeof b, "%.9E", (double)(c.ranlux_int_max + 1ull));
        o << "#define FS_RIM " << b << "f\n";  // kernel.py:334: always a float literal
    }
    if (c.enable_bins) {
        o << "#define FS_XMIN " << lit(c.x_min) << "\n#define FS_XMAX " << lit(c.x_max)
          << "\n#define FS_BINRES " << c.bin_resolution_per_dof << "\n#define FS_INVBIN "
          << lit((double)c.bin_resolution_per_dof / (c.x_max - c.x_min)) << "\n";
    }
    if (nhist) {
        o << "#define FS_HLO " << lit(c.hist_lo) << "\n#define FS_HHI " << lit(c.hist_hi)
          << "\n#define FS_HBINS " << c.hist_bins << "\n#define FS_HINVW "
          << lit((double)c.hist_bins / (c.hist_hi - c.hist_lo)) << "\n";
    } else {
        o << "#define FS_HBINS 0\n";
    }
    o << "#define eps FS_EPS\n";  // kernel.c:31
    o << sigma_table(c.bisection_level, c.beta / (double)c.n_slices, dbl);
    o << "\n// ---- random number generators ----\n" << kRngSrc << "\n";
    if (c.learned) o << "\n// ---- learned proposal network ----\n" << kMlpSrc << "\n";
    o << "\n// ---- plugin userCode ----\n" << cvt(user_code) << "\n";
    std::ostringstream args, at;
    for (int i = 0; i < c.dof; i++) {
        args << (i ? ", " : "") << "FT x" << (i + 1);
        at << (i ? ", " : "") << "FS_AT(P, " << i << ", (i))";
    }
    o << "#define FS_ARGS_AT(P, i) " << at.str() << "\n";
    // Plugins of more than 8 DOF (clusters of 4+ atoms, tens of pair terms) are called, not
    // inlined: the sweep evaluates the potential at several places, and inlined copies of a
    // 45-pair potential overflow the instruction cache (measured: +19% to +47% on a 10-atom
    // cluster).
    const char *inl = c.dof > 8 ? "__device__ __noinline__ " : "__device__ __forceinline__ ";
    o << inl << "FT fs_pot(" << args.str() << ") { return (" << cvt(potential)
      << "); }\n";
    auto fn = [&](const char *name, const std::vector<std::string> &ex) {
        if (ex.empty()) return;
        o << inl << "void " << name << "(" << args.str() << ", FT *o) {\n";
        for (size_t i = 0; i < ex.size(); i++) o << "    o[" << i << "] = (" << cvt(ex[i]) << ");\n";
        o << "}\n";
    };
    fn("fs_ops", h.ops);
    fn("fs_cors", h.cors);
    if (nhist) fn("fs_hist", h.hists);
    o << "\n// ---- sweep kernel ----\n" << kPimcSrc << "\n";
    return o.str();
}

// ------------------------------------------------------------------ NVRTC + cache
static int compile_module(fs_handle *h, const std::string &src, bool fast, std::string *cubin, std::string *log);

// internal entry points for the library's other translation units (not exported)
__attribute__((visibility("hidden"))) std::string fsi_float_literals(const std::string &s) { return float_literals(s); }
__attribute__((visibility("hidden"))) std::string fsi_prelude(bool dbl) { return gen_prelude(dbl); }
__attribute__((visibility("hidden"))) const char *fsi_rng_src() { return kRngSrc; }
__attribute__((visibility("hidden"))) int fsi_nskip_for(int lux) { return nskip_for(lux); }
__attribute__((visibility("hidden"))) const char *fsi_batch_src();
__attribute__((visibility("hidden"))) int fsi_compile(const std::string &src, bool fast, std::string *cubin,
                                                      std::string *log)
{
    fs_handle tmp;
    int rc = compile_module(&tmp, src, fast, cubin, log);
    if (rc) g_thread_err = tmp.err;
    return rc;
}
static std::mutex g_cache_mu;
static std::unordered_map<std::string, std::string> g_cubins;

static uint64_t fnv1a(const std::string &s, uint64_t hsh = 1469598103934665603ull)
{
    for (unsigned char ch : s) {
        hsh ^= ch;
        hsh *= 1099511628211ull;
    }
    return hsh;
}

static std::string cache_dir()
{
    const char *d = std::getenv("FS_CACHE_DIR");
    if (d && *d) return d;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/feynsimul_gb300";
}

static int compile_module(fs_handle *h, const std::string &src, bool fast, std::string *cubin,
                          std::string *log)
{
    std::vector<std::string> opts = {"--gpu-architecture=sm_103a", "-default-device", "--std=c++17",
                                      "-lineinfo", "--ptxas-options=-v"};
    if (fast)
        opts.push_back("--use_fast_math");
    else
        opts.push_back("--fmad=false");
    std::string key_text = src;
    for (auto &s : opts) key_text += "\n" + s;
    char keybuf[64];
    snprintf(keybuf, sizeof keybuf, "%016llx%016llx", (unsigned long long)fnv1a(key_text),
             (unsigned long long)fnv1a(key_text, 0x9E3779B97F4A7C15ull));
    const std::string key = keybuf;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        auto it = g_cubins.find(key);
        if (it != g_cubins.end()) {
            *cubin = it->second;
            *log = "(cached)";
            return FS_OK;
        }
    }
    const std::string path = cache_dir() + "/" + key + ".cubin";
    {
        std::ifstream f(path, std::ios::binary);
        if (f) {
            std::stringstream ss;
            ss << f.rdbuf();
            *cubin = ss.str();
            if (!cubin->empty()) {
                std::ifstream lf(path + ".log");
                std::stringstream ls;
                if (lf) ls << lf.rdbuf();
                *log = "(disk cache " + path + ")\n" + ls.str();
                std::lock_guard<std::mutex> lk(g_cache_mu);
                g_cubins[key] = *cubin;
                return FS_OK;
            }
        }
    }
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, src.c_str(), "feynsimul_sweep.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
        return fail(h, FS_ERR_COMPILE, "nvrtcCreateProgram failed");
    std::vector<const char *> copts;
    for (auto &s : opts) copts.push_back(s.c_str());
    nvrtcResult r = nvrtcCompileProgram(prog, (int)copts.size(), copts.data());
    size_t lsz = 0;
    nvrtcGetProgramLogSize(prog, &lsz);
    log->assign(lsz, '\0');
    if (lsz) nvrtcGetProgramLog(prog, &(*log)[0]);
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return fail(h, FS_ERR_COMPILE, "NVRTC compilation failed: %s\n%s", nvrtcGetErrorString(r),
                    log->substr(0, 1800).c_str());
    }
    size_t csz = 0;
    nvrtcGetCUBINSize(prog, &csz);
    cubin->assign(csz, '\0');
    nvrtcGetCUBIN(prog, &(*cubin)[0]);
    nvrtcDestroyProgram(&prog);
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        g_cubins[key] = *cubin;
    }
    // best-effort disk cache: write a temporary file, then rename it into place
    std::string dir = cache_dir();
    for (size_t p = 1; p <= dir.size(); p++)
        if (p == dir.size() || dir[p] == '/') ::mkdir(dir.substr(0, p).c_str(), 0755);
    std::string tmp = path + "." + std::to_string((long long)::getpid()) + ".tmp";
    {
        std::ofstream f(tmp, std::ios::binary);
        if (f) f.write(cubin->data(), (std::streamsize)cubin->size());
    }
    {
        std::ofstream lf(tmp + ".log");
        if (lf) lf << *log;
    }
    std::rename((tmp + ".log").c_str(), (path + ".log").c_str());
    std::rename(tmp.c_str(), path.c_str());
    return FS_OK;
}

static int load_module(fs_handle *h, const std::string &cubin)
{
    CUDA_TRY(h, cudaLibraryLoadData(&h->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0),
             FS_ERR_CUDA);
    return FS_OK;
}

// ------------------------------------------------------------------ validation
// The checks of kernel.py:93-211 that concern the device path; the Python layer raises the
// reference's exception types before it gets here.
// SMs of the current device (152 on a GB300, also the answer without a device, for
// compile-only use)
static int device_sms()
{
    static const int sms = [] {
        int dev = 0, n = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
            return n;
        (void)cudaGetLastError();
        return 152;
    }();
    return sms;
}

static int validate(const fs_config &c, int nops, int ncor, int nhist)
{
    if (c.dof < 1 || c.dof > 256) return fail(nullptr, FS_ERR_CONFIG, "DOF must be in [1, 256]");
    if (c.n_slices < 2 || (c.n_slices & (c.n_slices - 1)))
        return fail(nullptr, FS_ERR_CONFIG, "Path node number, N, must be a power of 2.");
    if (c.bisection_level < 0 || (1ll << c.bisection_level) > c.n_slices)
        return fail(nullptr, FS_ERR_CONFIG, "2^S must be less than or equal to N.");
    if (!(c.beta > 0.0) || !std::isfinite(c.beta)) return fail(nullptr, FS_ERR_CONFIG, "beta must be a positive float");
    if (c.n_walkers < 1) return fail(nullptr, FS_ERR_CONFIG, "nbrOfWalkers must be >= 1");
    if (c.walkers_per_group < 1 || c.n_walkers % c.walkers_per_group)
        return fail(nullptr, FS_ERR_CONFIG,
                    "The number of walkers must be a multiple of the number of walkers per work group.");
    if (c.operator_runs < 1 || c.metro_steps_per_operator_run < 0)
        return fail(nullptr, FS_ERR_CONFIG, "operatorRuns must be >= 1 and metroStepsPerOperatorRun >= 0");
    if (c.enable_parallelize_path && (c.n_slices >> c.bisection_level) > 1024)
        return fail(nullptr, FS_ERR_CONFIG, "N / 2^S threads per walker must not exceed 1024");
    if (c.enable_ranlux) {
        int lux = c.luxury_factor + 1;
        int ns = nskip_for(lux);
        if (c.luxury_factor < 0 || (lux > 4 && lux < 24) || ns % 4 != 0 || (ns != 0 && ns < 24))
            return fail(nullptr, FS_ERR_CONFIG, "luxuaryFactor needs to be an uint >= 0 (0-3, or >= 23 with p-24 a multiple of 4).");
        if (c.ranlux_int_max < 1 || c.ranlux_int_max > 0xFFFFFFFFull)
            return fail(nullptr, FS_ERR_CONFIG, "ranluxIntMax needs to be an uint > 0.");
    }
    if (c.enable_bins) {
        if (c.bin_resolution_per_dof < 1 || !(c.x_max > c.x_min))
            return fail(nullptr, FS_ERR_CONFIG, "xMin < xMax and binResolutionPerDOF >= 1 are needed when enableBins is True.");
        double nb = std::pow((double)c.bin_resolution_per_dof, c.dof);
        if (nb > 1e9) return fail(nullptr, FS_ERR_CONFIG, "binResolutionPerDOF ** DOF bins is too large");
    }
    if (nhist > 0 && (c.hist_bins < 1 || c.hist_bins > 16384 || !(c.hist_hi > c.hist_lo)))
        return fail(nullptr, FS_ERR_CONFIG, "histogram needs 1..16384 bins and hist_lo < hist_hi");
    if (c.accum < 0 || c.accum > 3) return fail(nullptr, FS_ERR_CONFIG, "accum must be 0..3");
    if (c.potential_cache < 0 || c.potential_cache > 3)
        return fail(nullptr, FS_ERR_CONFIG, "potential_cache must be 0..3");
    if (c.partials != FS_PARTIALS_FP32 && c.partials != FS_PARTIALS_EXACT)
        return fail(nullptr, FS_ERR_CONFIG, "partials must be 0 (FP32) or 1 (exact)");
    if (nops < 0 || ncor < 0 || nops > 64 || ncor > 16)
        return fail(nullptr, FS_ERR_CONFIG, "at most 64 operators and 16 correlators");
    if (c.walkers_per_block < 0) return fail(nullptr, FS_ERR_CONFIG, "walkers_per_block must be >= 0");
    if (c.learned) {
        if (!c.enable_parallelize_path || c.dof > 8 || c.bisection_level < 1 || c.enable_double)
            return fail(nullptr, FS_ERR_CONFIG,
                        "the learned proposal needs parallel-path mode, FP32, DOF <= 8 and S >= 1");
        if ((c.n_slices >> c.bisection_level) > 32)
            return fail(nullptr, FS_ERR_CONFIG, "the learned proposal needs N / 2^S <= 32");
    }
    if (c.min_blocks_per_sm < 0 || c.min_blocks_per_sm > 32)
        return fail(nullptr, FS_ERR_CONFIG, "min_blocks_per_sm must be in [0, 32]");
    if (c.moves < 0 || c.moves > 7) return fail(nullptr, FS_ERR_CONFIG, "moves must be a mask of FS_MOVE_*");
    if (c.enable_parallelize_path && (c.moves & FS_MOVE_SINGLE_NODE))
        return fail(nullptr, FS_ERR_CONFIG, "Single node move not possible when enableParallelizePath is True.");
    if (c.enable_parallelize_path && (c.moves & FS_MOVE_PATH_SHIFT))
        return fail(nullptr, FS_ERR_CONFIG, "Shift path not possible when enableParallelizePath is True.");
    if (c.enable_parallelize_path && c.moves && !(c.moves & FS_MOVE_BISECTION))
        return fail(nullptr, FS_ERR_CONFIG, "parallel-path mode needs the bisection move");
    if (c.learned && c.moves && c.moves != FS_MOVE_BISECTION)
        return fail(nullptr, FS_ERR_CONFIG, "the learned proposal goes with the bisection move only");
    return FS_OK;
}

static void free_buffers(fs_handle *h)
{
    void *bufs[] = {h->d_paths, h->d_accepts, h->d_seeds, h->d_snap, h->d_wseeds, h->d_rtab,
                    h->d_gtab, h->d_bins, h->d_ops, h->d_cor, h->d_hist, h->d_status,
                    h->d_mlp_frag, h->d_mlp_bias, h->d_red, h->d_shift_old, h->d_wops, h->d_vcache};
    for (void *p : bufs)
        if (p) cudaFree(p);
}

static int dalloc(fs_handle *h, void **p, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(h, FS_ERR_OOM, "Unable to allocate global memory on device, out of memory? (%zu bytes: %s)",
                    bytes, cudaGetErrorString(e));
    }
    CUDA_TRY(h, cudaMemsetAsync(*p, 0, bytes, h->stream), FS_ERR_CUDA);
    h->device_bytes += bytes;
    return FS_OK;
}

// Host-only half of fs_create: validation, geometry, source generation, NVRTC compile.
static int prepare(const fs_config *cfg, const char *potential, const char *user_code,
                   const char *const *operators, int32_t n_operators, const char *const *correlators,
                   int32_t n_correlators, const char *const *histograms, int32_t n_histograms,
                   fs_handle **out, std::string *cubin_out)
{
    if (!cfg || !potential || !out) return fail(nullptr, FS_ERR_CONFIG, "null argument");
    *out = nullptr;
    int rc = validate(*cfg, n_operators, n_correlators, n_histograms);
    if (rc) return rc;
    fs_handle *h = new fs_handle();
    h->cfg = *cfg;
    const fs_config &c = h->cfg;
    for (int i = 0; i < n_operators; i++) h->ops.push_back(operators[i] ? operators[i] : "0");
    for (int i = 0; i < n_correlators; i++) h->cors.push_back(correlators[i] ? correlators[i] : "1");
    if (c.hist_bins > 0)
        for (int i = 0; i < n_histograms; i++) h->hists.push_back(histograms[i] ? histograms[i] : "0");

    // ---- geometry (kernel.py:192-211) ----
    h->seg = 1 << c.bisection_level;
    h->tpw = c.enable_parallelize_path ? (c.n_slices >> c.bisection_level) : 1;
    h->n_threads = (long long)c.n_walkers * h->tpw;
    h->ft = c.enable_double ? 8 : 4;
    {
        // FP32-partial correlator sums (every mode but the reference's FP32 order, FP32
        // builds) with at most 4 lags per thread run every lag in one pass over the slice
        // values, stored twice in a row so that slice s1 + tau needs no wrap.
        // Correlator helpers: a walker of at most 32 segment threads gets extra threads for
        // the lag sums, up to 64 lag threads per walker (FS_MX in fs_pimc.cuh).  They need
        // every CTA full (the walker count a multiple of the walkers per CTA, chosen below).
        // Where the movers of a CTA fill whole warps (walker count and walkers per CTA
        // multiples of 32 / threads per walker) the helpers are pipelined (FS_PIPE): the
        // movers copy their slices to a double-buffered path snapshot, and the helpers alone
        // evaluate the correlator values on it and sum the lags, one measurement behind the
        // moves.
        // The pipelined helpers give each thread 4 consecutive lags (N/8 lag threads per
        // walker) and sum FP32 partials over the doubled slice values.
        if (!h->cors.empty() && c.enable_parallelize_path && !c.global_path && !c.learned && h->tpw <= 32) {
            const int lag_threads = std::min(c.n_slices / 2, 64);
            const int wpw = 32 / h->tpw;
            const int wpb_min = c.walkers_per_block > 0 ? c.walkers_per_block : wpw;
            const int groups = (c.n_slices / 8 + h->tpw - 1) / h->tpw;
            const bool fma_partials = (c.accum == FS_ACCUM_FP64 || c.accum == FS_ACCUM_KAHAN) &&
                                      !c.enable_double && c.partials == FS_PARTIALS_FP32;
            if (fma_partials && c.n_slices % 8 == 0 && c.n_slices >= 16 && h->tpw >= 2 && c.n_walkers % wpw == 0 &&
                wpb_min % wpw == 0 && c.n_walkers % wpb_min == 0 &&
                (long long)wpb_min * h->tpw * (1 + groups) <= 512) {
                h->pipe = 1;
                h->mx = 1 + groups;
            } else if (lag_threads > h->tpw) {
                h->mx = lag_threads / h->tpw;
            }
            if (c.walkers_per_block > 0 && c.n_walkers % c.walkers_per_block) h->mx = 1, h->pipe = 0;
        }
        const long long lag_tpw = (long long)h->tpw * (h->mx - h->pipe);
        const long long lpt = h->pipe ? 4 : (c.n_slices / 2 + lag_tpw - 1) / lag_tpw;
        h->cor_ilv = (c.accum != 0 && !c.enable_double && lpt <= 4) ? 1 : 0;
        // per-walker stride an odd multiple of 64 bytes: two walkers sharing a warp read
        // opposite bank halves
        const long long q = 64 / (long long)h->ft;
        long long cw = (long long)h->cors.size() * c.n_slices * (h->cor_ilv ? 2 : 1);
        if (h->pipe) {
            // two path snapshots in the padded slice layout, 16-word multiples (FS_SNSTRIDE)
            const long long dstr = c.n_slices + (c.n_slices >> c.bisection_level);
            h->snstride = ((c.dof * dstr + 15) / 16) * 16;
            cw += 2 * h->snstride;
        }
        if (cw) {
            cw = ((cw + q - 1) / q) * q;
            if ((cw / q) % 2 == 0) cw += q;
        }
        h->cwstride = cw;
    }
    // padded shared-memory path (see FS_PHYS in fs_pimc.cuh): one word after every 2^S
    // slices; the walker stride is an odd multiple of 16 words
    const long long dstride = c.n_slices + (c.n_slices >> c.bisection_level);
    long long wstride = (long long)c.dof * dstride;
    wstride = ((wstride + 15) / 16) * 16;
    if ((wstride / 16) % 2 == 0) wstride += 16;
    if (c.global_path) wstride = (long long)c.dof * c.n_slices;  // no shared-memory path
    h->wstride = wstride;
    // potential cache: one value per slice in the path's padded slice layout, walker stride
    // an odd multiple of 16 words
    long long vstride = ((dstride + 15) / 16) * 16;
    if ((vstride / 16) % 2 == 0) vstride += 16;
    const size_t per_walker_base =
        (size_t)((c.global_path ? 0 : wstride) + h->cwstride) * h->ft;
    // the path-shift and single-node moves change slices outside the bisection's
    // bookkeeping, so they go without the potential cache
    const bool other_moves = (c.moves & (FS_MOVE_PATH_SHIFT | FS_MOVE_SINGLE_NODE)) != 0;
    h->vstride = (c.potential_cache == 2 || c.potential_cache == 3 || other_moves) ? 0 : vstride;
    h->vglobal = c.potential_cache == 3 && !other_moves ? 1 : 0;
    size_t per_walker = per_walker_base + (size_t)h->vstride * h->ft;
    const size_t hist_bytes = (size_t)(c.hist_bins > 0 && !h->hists.empty() ? c.hist_bins : 0) * 4;
    if (c.walkers_per_block > 0) {
        h->wpb = c.walkers_per_block;
    } else if (h->mx > 1) {
        // CTAs of about 128 threads (moving and summing), every CTA full; pipelined: the
        // movers in whole warps
        // pipelined: the movers in whole warps, as few walkers per CTA as that allows (the
        // CTAs spread evenly over the SMs)
        const int step = h->pipe ? 32 / h->tpw : 1;
        h->wpb = h->pipe ? step : std::max(1, 128 / (h->tpw * h->mx));
        while (h->wpb > step && (c.n_walkers % h->wpb || per_walker * h->wpb + hist_bytes > 100 * 1024))
            h->wpb -= step;
    } else if (h->tpw > 32) {
        h->wpb = 1;
    } else {
        int target = h->tpw == 1 ? 64 : 128;
        h->wpb = std::max(1, target / h->tpw);
        while (h->wpb > 1 && per_walker * h->wpb + hist_bytes > 100 * 1024) h->wpb /= 2;
    }
    h->wpb = std::min(h->wpb, c.n_walkers);
    if (h->tpw > 32 && h->wpb != 1) {
        delete h;
        return fail(nullptr, FS_ERR_CONFIG, "walkers_per_block must be 1 when N / 2^S > 32");
    }
    if (h->tpw <= 32 && 32 % h->tpw != 0) {
        delete h;
        return fail(nullptr, FS_ERR_CONFIG, "internal: threads per walker must divide 32");
    }
    if (c.learned) {
        // the network is evaluated warp-wide: every lane of every warp must hold a walker
        const int wpw = 32 / h->tpw;
        h->wpb = std::max(wpw, (h->wpb / wpw) * wpw);
        if (c.n_walkers % wpw) {
            delete h;
            return fail(nullptr, FS_ERR_CONFIG, "the learned proposal needs the walker count to be a multiple of %d", wpw);
        }
        while (c.n_walkers % h->wpb) h->wpb -= wpw;
    }
    h->block = h->wpb * h->tpw * h->mx;
    if (h->block > 1024) {
        delete h;
        return fail(nullptr, FS_ERR_CONFIG, "walkers_per_block * threads per walker exceeds 1024");
    }
    h->grid = (c.n_walkers + h->wpb - 1) / h->wpb;
    h->smem = per_walker * h->wpb + hist_bytes;
    if (h->vstride && c.potential_cache == 0) {
        // automatic: the cache halves the potential evaluations but takes shared memory;
        // keep it where it costs no resident CTA per SM, or where the potential is large
        // (more than 8 DOF: a cluster of 4+ atoms)
        auto ctas = [](size_t smem) { return (227ll * 1024) / (long long)(smem + 1024); };
        const size_t without = per_walker_base * h->wpb + hist_bytes;
        if (ctas(h->smem) < std::min(ctas(without), 2048ll / h->block) && c.dof <= 8) h->vstride = 0;
    }
    if (h->smem > 227 * 1024 && h->vstride && c.potential_cache != 1) h->vstride = 0;  // no room
    if (!h->vstride) {
        per_walker = per_walker_base;
        h->smem = per_walker * h->wpb + hist_bytes;
        // automatic: where shared memory has no room for the cache, keep it in device memory
        // (L1/L2), for potentials of 3 or more DOF and launches of more than one move; the
        // launch starts with one potential evaluation per slice
        if (c.potential_cache == 0 && !other_moves && c.dof >= 3 &&
            (long long)c.operator_runs * c.metro_steps_per_operator_run >= 2)
            h->vglobal = 1;
    }
    // Register budget: unless the caller fixes it, compile for as many CTAs per SM as shared
    // memory admits (<= 2048 threads per SM, >= 64 registers per thread) and as the grid can
    // put on one SM.  Without the bound the compiler spends registers freely and the large
    // kernels drop to one CTA per SM; a grid of at most one CTA per SM gets every register.
    if (h->cfg.min_blocks_per_sm == 0) {
        long long by_smem = (227ll * 1024) / std::max<long long>(1, (long long)h->smem + 1024);
        long long by_threads = 2048 / h->block;
        long long by_regs = 65536 / (64ll * h->block);
        long long by_grid = (h->grid + device_sms() - 1) / device_sms();
        h->cfg.min_blocks_per_sm =
            (int)std::max(1ll, std::min(std::min(std::min(by_smem, by_threads), by_regs), by_grid));
    }
    if (h->smem > 227 * 1024) {
        delete h;
        return fail(nullptr, FS_ERR_CONFIG,
                    "a walker's path does not fit in shared memory (%zu bytes per CTA); lower walkers_per_block",
                    h->smem);
    }

    // ---- source + compile ----
    h->source = gen_source(*h, potential, user_code ? user_code : "");
    rc = compile_module(h, h->source, c.fast_math != 0, cubin_out, &h->log);
    if (rc) {
        g_thread_err = h->err;
        delete h;
        return rc;
    }
    *out = h;
    return FS_OK;
}

extern "C" int fs_compile_only(const fs_config *cfg, const char *potential, const char *user_code,
                               const char *const *operators, int32_t n_operators,
                               const char *const *correlators, int32_t n_correlators,
                               const char *const *histograms, int32_t n_histograms, char *log,
                               size_t log_capacity)
{
    fs_handle *h = nullptr;
    std::string cubin;
    int rc = prepare(cfg, potential, user_code, operators, n_operators, correlators, n_correlators,
                     histograms, n_histograms, &h, &cubin);
    std::string text = rc ? g_thread_err : h->log;
    if (log && log_capacity) {
        size_t k = std::min(log_capacity - 1, text.size());
        memcpy(log, text.data(), k);
        log[k] = 0;
    }
    delete h;
    return rc;
}

extern "C" int fs_create(const fs_config *cfg, const char *potential, const char *user_code,
                         const char *const *operators, int32_t n_operators,
                         const char *const *correlators, int32_t n_correlators,
                         const char *const *histograms, int32_t n_histograms, fs_handle **out)
{
    fs_handle *h = nullptr;
    std::string cubin;
    int rc = prepare(cfg, potential, user_code, operators, n_operators, correlators, n_correlators,
                     histograms, n_histograms, &h, &cubin);
    if (rc) return rc;
    const fs_config &c = h->cfg;
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) {
        fail(nullptr, FS_ERR_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
        delete h;
        return FS_ERR_CUDA;
    }
#define CREATE_TRY(call)                                      \
    do {                                                      \
        int r_ = (call);                                      \
        if (r_) {                                             \
            g_thread_err = h->err;                            \
            free_buffers(h);                                  \
            if (h->lib) cudaLibraryUnload(h->lib);            \
            if (h->stream) cudaStreamDestroy(h->stream);      \
            delete h;                                         \
            return r_;                                        \
        }                                                     \
    } while (0)
    auto cu = [&](cudaError_t err, const char *what) -> int {
        if (err != cudaSuccess) return fail(h, FS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(err));
        return FS_OK;
    };
    CREATE_TRY(cu(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "cudaStreamCreate"));
    CREATE_TRY(cu(cudaEventCreate(&h->ev0), "cudaEventCreate"));
    CREATE_TRY(cu(cudaEventCreate(&h->ev1), "cudaEventCreate"));
    CREATE_TRY(load_module(h, cubin));
    CREATE_TRY(cu(cudaLibraryGetKernel(&h->k_metro, h->lib, "fs_metropolis"), "fs_metropolis"));
    CREATE_TRY(cu(cudaLibraryGetKernel(&h->k_rinit, h->lib, "fs_ranlux_init"), "fs_ranlux_init"));
    CREATE_TRY(cu(cudaFuncSetAttribute((const void *)h->k_metro, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)h->smem), "cudaFuncSetAttribute"));
    {
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, (const void *)h->k_metro) == cudaSuccess) h->regs = fa.numRegs;
        else cudaGetLastError();
    }

    // ---- buffers (kernel.py:386-457) ----
    const size_t W = c.n_walkers, T = h->n_threads, N = c.n_slices;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) cudaGetLastError();
    h->op_elem = c.accum == 0 ? h->ft : (c.accum == 2 ? 4 : 8);
    h->n_ops_elems = T * h->ops.size() * (c.accum == 3 ? 3 : 1);
    h->cor_elem = c.accum == 0 ? h->ft : (c.accum == 3 ? 24 : 8);
    h->n_cor_lags = W * h->cors.size() * (N / 2);
    h->n_cor_elems = h->n_cor_lags * (c.accum == 3 ? 4 : 1);
    h->n_bins = c.enable_bins ? (size_t)std::llround(std::pow((double)c.bin_resolution_per_dof, c.dof)) : 0;
    h->n_hist = h->hists.empty() ? 0 : (size_t)c.hist_bins;
    h->g_rows = c.compat ? T : W;
    size_t need = W * c.dof * N * h->ft + T * 4 + h->n_ops_elems * h->op_elem + h->n_cor_lags * h->cor_elem +
                  h->n_bins * 4 + h->n_hist * 8 +
                  (c.enable_ranlux ? (T + h->g_rows) * 112 : ((T + 1) * 16 * 2 + W * 16));
    if (free_b && need > free_b) {
        fail(nullptr, FS_ERR_OOM,
             "Unable to allocate global memory on device, out of memory? (need %zu bytes, %zu free)", need, free_b);
        cudaStreamDestroy(h->stream);
        cudaLibraryUnload(h->lib);
        delete h;
        return FS_ERR_OOM;
    }
    CREATE_TRY(dalloc(h, &h->d_paths, W * c.dof * N * h->ft));
    CREATE_TRY(dalloc(h, (void **)&h->d_accepts, T * 4));
    if (c.enable_ranlux) {
        CREATE_TRY(dalloc(h, (void **)&h->d_rtab, T * 112));
        CREATE_TRY(dalloc(h, (void **)&h->d_gtab, h->g_rows * 112));
    } else {
        CREATE_TRY(dalloc(h, (void **)&h->d_seeds, (T + 1) * 16));
        if (c.compat) CREATE_TRY(dalloc(h, (void **)&h->d_snap, (T + 1) * 16));
        CREATE_TRY(dalloc(h, (void **)&h->d_wseeds, W * 16));
    }
    CREATE_TRY(dalloc(h, &h->d_ops, h->n_ops_elems * h->op_elem));
    CREATE_TRY(dalloc(h, &h->d_cor, h->n_cor_lags * h->cor_elem));
    CREATE_TRY(dalloc(h, (void **)&h->d_bins, h->n_bins * 4));
    CREATE_TRY(dalloc(h, (void **)&h->d_hist, h->n_hist * 8));
    CREATE_TRY(dalloc(h, (void **)&h->d_status, 16));
    if ((c.moves & FS_MOVE_PATH_SHIFT) && !c.compat) CREATE_TRY(dalloc(h, &h->d_shift_old, W * N * h->ft));
    if (h->vglobal) CREATE_TRY(dalloc(h, &h->d_vcache, W * N * h->ft));
    if (c.learned) {
        CREATE_TRY(dalloc(h, &h->d_mlp_frag, (size_t)FS_MLP_FRAG_BYTES));
        CREATE_TRY(dalloc(h, (void **)&h->d_mlp_bias, (size_t)FS_MLP_NBIAS_FLOATS * 4));
    }
    CREATE_TRY(cu(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize"));
#undef CREATE_TRY
    *out = h;
    return FS_OK;
}

extern "C" int fs_destroy(fs_handle *h)
{
    if (!h) return FS_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_buffers(h);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    for (cudaEvent_t e : h->ev_chunk) cudaEventDestroy(e);
    if (h->s_in) cudaStreamDestroy(h->s_in);
    if (h->s_out) cudaStreamDestroy(h->s_out);
    if (h->s_comp2) cudaStreamDestroy(h->s_comp2);
    if (h->lib) cudaLibraryUnload(h->lib);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return FS_OK;
}

extern "C" const char *fs_last_error(const fs_handle *h) { return h ? h->err.c_str() : g_thread_err.c_str(); }
extern "C" const char *fs_build_log(const fs_handle *h) { return h ? h->log.c_str() : ""; }
extern "C" const char *fs_source(const fs_handle *h) { return h ? h->source.c_str() : ""; }
extern "C" const char *fs_version(void) { return FS_VERSION; }

extern "C" int fs_query(const fs_handle *h, fs_info *info)
{
    if (!h || !info) return FS_ERR_CONFIG;
    info->n_threads = h->n_threads;
    info->threads_per_walker = h->tpw;
    info->walkers_per_block = h->wpb;
    info->block_threads = h->block;
    info->grid_blocks = h->grid;
    info->smem_bytes = (int64_t)h->smem;
    info->registers = h->regs;
    info->device_bytes = (int64_t)h->device_bytes;
    info->nodes_per_move = h->seg - 1;
    info->uniforms_per_move = 2ll * h->cfg.dof * (h->seg - 1) + 1;
    info->potential_cache = h->vglobal ? 3 : (h->vstride ? 1 : 0);
    return FS_OK;
}

// ------------------------------------------------------------------ host <-> device
static int copy_in(fs_handle *h, void *dst, const void *src, size_t bytes, size_t expect)
{
    if (!h) return FS_ERR_CONFIG;
    if (bytes != expect) return fail(h, FS_ERR_IO, "buffer has %zu bytes, expected %zu", bytes, expect);
    if (!dst) return fail(h, FS_ERR_STATE, "buffer not used by this configuration");
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    CUDA_TRY(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

static int copy_out(fs_handle *h, void *dst, const void *src, size_t bytes, size_t expect)
{
    if (!h) return FS_ERR_CONFIG;
    if (bytes != expect) return fail(h, FS_ERR_IO, "buffer has %zu bytes, expected %zu", bytes, expect);
    if (!src) return fail(h, FS_ERR_STATE, "buffer not used by this configuration");
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    CUDA_TRY(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

static size_t path_elems(const fs_handle *h) { return (size_t)h->cfg.n_walkers * h->cfg.dof * h->cfg.n_slices; }

extern "C" int fs_set_paths(fs_handle *h, const void *host, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_in(h, h->d_paths, host, n * h->ft, path_elems(h) * h->ft);
}
extern "C" int fs_get_paths(fs_handle *h, void *host, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, host, h->d_paths, n * h->ft, path_elems(h) * h->ft);
}
extern "C" int fs_set_xorshift_seeds(fs_handle *h, const uint32_t *rows, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_in(h, h->d_seeds, rows, n * 16, (h->n_threads + 1) * 16);
}
extern "C" int fs_get_xorshift_seeds(fs_handle *h, uint32_t *rows, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, rows, h->d_seeds, n * 16, (h->n_threads + 1) * 16);
}
extern "C" int fs_set_walker_seeds(fs_handle *h, const uint32_t *rows, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_in(h, h->d_wseeds, rows, n * 16, (size_t)h->cfg.n_walkers * 16);
}
extern "C" int fs_get_walker_seeds(fs_handle *h, uint32_t *rows, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, rows, h->d_wseeds, n * 16, (size_t)h->cfg.n_walkers * 16);
}

static int ranlux_seed_rows(fs_handle *h, uint32_t *tab, size_t rows, const uint64_t *xs, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    if (!tab) return fail(h, FS_ERR_STATE, "RANLUX is not enabled for this handle");
    if (n != rows) return fail(h, FS_ERR_IO, "got %zu seed values, expected %zu", n, rows);
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    void *d_xs = nullptr;
    CUDA_TRY(h, cudaMallocAsync(&d_xs, n * 8, h->stream), FS_ERR_OOM);
    CUDA_TRY(h, cudaMemcpyAsync(d_xs, xs, n * 8, cudaMemcpyHostToDevice, h->stream), FS_ERR_CUDA);
    int ni = (int)n;
    void *args[] = {&tab, &d_xs, &ni};
    CUDA_TRY(h, cudaLaunchKernel((const void *)h->k_rinit, dim3((unsigned)((n + 127) / 128)), dim3(128), args, 0,
                                 h->stream), FS_ERR_LAUNCH);
    CUDA_TRY(h, cudaFreeAsync(d_xs, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

extern "C" int fs_ranlux_init(fs_handle *h, const uint64_t *xs, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return ranlux_seed_rows(h, h->d_rtab, (size_t)h->n_threads, xs, n);
}
extern "C" int fs_ranlux_group_init(fs_handle *h, const uint64_t *xs, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return ranlux_seed_rows(h, h->d_gtab, h->g_rows, xs, n);
}
extern "C" int fs_get_ranlux_tables(fs_handle *h, uint32_t *tab, size_t nt, uint32_t *gtab, size_t ng)
{
    if (!h) return FS_ERR_CONFIG;
    int rc = FS_OK;
    if (tab) rc = copy_out(h, tab, h->d_rtab, nt * 112, (size_t)h->n_threads * 112);
    if (!rc && gtab) rc = copy_out(h, gtab, h->d_gtab, ng * 112, h->g_rows * 112);
    return rc;
}
extern "C" int fs_set_ranlux_tables(fs_handle *h, const uint32_t *tab, size_t nt, const uint32_t *gtab, size_t ng)
{
    if (!h) return FS_ERR_CONFIG;
    int rc = FS_OK;
    if (tab) rc = copy_in(h, h->d_rtab, tab, nt * 112, (size_t)h->n_threads * 112);
    if (!rc && gtab) rc = copy_in(h, h->d_gtab, gtab, ng * 112, h->g_rows * 112);
    return rc;
}

// ------------------------------------------------------------------ run
struct FsArgsHost {  // mirrors FsArgs in fs_pimc.cuh
    void *paths;
    uint32_t *accepts, *seeds;
    const uint32_t *seed_snap;
    uint32_t *walker_seeds, *rtab, *gtab;
    void *op_means, *cor_means;
    uint32_t *bins;
    unsigned long long *hist;
    int *status;
    double opnorm;
    void *shift_old;
    unsigned long long step_base;
    const void *mlp_frag;
    const float *mlp_bias;
    float mlp_inv_scale;
    int block_offset;
    void *vcache;
};

extern "C" int fs_get_step_counter(fs_handle *h, uint64_t *steps)
{
    if (!h || !steps) return FS_ERR_CONFIG;
    *steps = h->steps_done;
    return FS_OK;
}

extern "C" int fs_set_step_counter(fs_handle *h, uint64_t steps)
{
    if (!h) return FS_ERR_CONFIG;
    h->steps_done = steps;
    return FS_OK;
}

extern "C" int fs_set_learned_proposal(fs_handle *h, const void *frag, size_t frag_bytes, const float *bias,
                                       size_t n_bias, double inv_scale)
{
    if (!h) return FS_ERR_CONFIG;
    if (!h->d_mlp_frag) return fail(h, FS_ERR_STATE, "handle was created without the learned proposal");
    int rc = copy_in(h, h->d_mlp_frag, frag, frag_bytes, (size_t)FS_MLP_FRAG_BYTES);
    if (!rc) rc = copy_in(h, h->d_mlp_bias, bias, n_bias * 4, (size_t)FS_MLP_NBIAS_FLOATS * 4);
    if (!rc) h->mlp_inv_scale = inv_scale;
    return rc;
}

static void fill_args(fs_handle *h, FsArgsHost &a);

extern "C" int fs_run(fs_handle *h, int32_t n_launches)
{
    if (!h) return FS_ERR_CONFIG;
    if (n_launches < 1) return fail(h, FS_ERR_CONFIG, "n_launches must be >= 1");
    const fs_config &c = h->cfg;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    FsArgsHost a;
    fill_args(h, a);
    void *args[] = {&a};
    CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), FS_ERR_CUDA);
    for (int i = 0; i < n_launches; i++) {
        a.step_base = h->steps_done;  // copied at launch
        h->steps_done += (unsigned long long)c.operator_runs * c.metro_steps_per_operator_run;
        if (h->d_snap)
            CUDA_TRY(h, cudaMemcpyAsync(h->d_snap, h->d_seeds, (h->n_threads + 1) * 16, cudaMemcpyDeviceToDevice,
                                        h->stream), FS_ERR_CUDA);
        CUDA_TRY(h, cudaLaunchKernel((const void *)h->k_metro, dim3(h->grid), dim3(h->block), args, h->smem, h->stream),
                 FS_ERR_LAUNCH);
    }
    CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream), FS_ERR_CUDA);
    h->timed = true;
    h->status_pending = true;
    return FS_OK;
}

// Pipelined run on host path buffers: the walkers are split into n_chunks CTA-aligned
// chunks; chunk c's paths are copied in on one stream, its n_launches sweeps run on the
// handle's stream as soon as they have arrived, and its paths are copied out on a third
// stream while later chunks compute.  Walkers are independent, so this equals
// set_paths + run + get_paths bit for bit (the reference-compatible xorshift mode, whose
// walker streams read other walkers' seed rows, runs as one chunk).
extern "C" int fs_run_host(fs_handle *h, const void *paths_in, void *paths_out, int32_t n_launches,
                           int32_t n_chunks)
{
    if (!h || !paths_in || !paths_out) return FS_ERR_CONFIG;
    if (n_launches < 1 || n_chunks < 0) return fail(h, FS_ERR_CONFIG, "n_launches must be >= 1, n_chunks >= 0");
    const fs_config &c = h->cfg;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    if (n_chunks == 0) {
        // automatic: as many chunks (up to 4) as still give every chunk half a wave of
        // resident CTAs; small grids run as one chunk
        if (!h->resident_per_sm) {
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)h->k_metro, h->block, h->smem) !=
                cudaSuccess)
                cudaGetLastError();
            h->resident_per_sm = std::max(per_sm, 1);
        }
        const long long half_wave = std::max(1ll, (long long)h->resident_per_sm * device_sms() / 2);
        n_chunks = (int)std::max(1ll, std::min(4ll, (long long)h->grid / half_wave));
    }
    if (h->d_snap) n_chunks = 1;
    n_chunks = std::min(n_chunks, std::min(h->grid, 64));
    h->last_chunks = n_chunks;
    FsArgsHost a;
    fill_args(h, a);
    void *args[] = {&a};
    const size_t bpw = (size_t)c.dof * c.n_slices * h->ft;
    const unsigned long long per_launch = (unsigned long long)c.operator_runs * c.metro_steps_per_operator_run;
    if (n_chunks == 1) {
        // one chunk: copy in, sweeps and copy out in the handle's stream order, no events
        const size_t bytes = (size_t)c.n_walkers * bpw;
        CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), FS_ERR_CUDA);
        CUDA_TRY(h, cudaMemcpyAsync(h->d_paths, paths_in, bytes, cudaMemcpyHostToDevice, h->stream), FS_ERR_CUDA);
        a.block_offset = 0;
        for (int i = 0; i < n_launches; i++) {
            a.step_base = h->steps_done + per_launch * (unsigned long long)i;
            if (h->d_snap)
                CUDA_TRY(h, cudaMemcpyAsync(h->d_snap, h->d_seeds, (h->n_threads + 1) * 16, cudaMemcpyDeviceToDevice,
                                            h->stream), FS_ERR_CUDA);
            CUDA_TRY(h, cudaLaunchKernel((const void *)h->k_metro, dim3(h->grid), dim3(h->block), args, h->smem,
                                         h->stream), FS_ERR_LAUNCH);
        }
        CUDA_TRY(h, cudaMemcpyAsync(paths_out, h->d_paths, bytes, cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
        h->steps_done += per_launch * (unsigned long long)n_launches;
        CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream), FS_ERR_CUDA);
        h->timed = true;
        h->status_pending = true;
        return FS_OK;
    }
    if (!h->s_in) CUDA_TRY(h, cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking), FS_ERR_CUDA);
    if (!h->s_out) CUDA_TRY(h, cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking), FS_ERR_CUDA);
    if (!h->s_comp2) CUDA_TRY(h, cudaStreamCreateWithFlags(&h->s_comp2, cudaStreamNonBlocking), FS_ERR_CUDA);
    while ((int)h->ev_chunk.size() < 2 * n_chunks + 2) {
        cudaEvent_t e;
        CUDA_TRY(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), FS_ERR_CUDA);
        h->ev_chunk.push_back(e);
    }
    CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream), FS_ERR_CUDA);
    // the copy streams start after everything queued before this call
    CUDA_TRY(h, cudaStreamWaitEvent(h->s_in, h->ev0, 0), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamWaitEvent(h->s_out, h->ev0, 0), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamWaitEvent(h->s_comp2, h->ev0, 0), FS_ERR_CUDA);
    // chunks alternate between two compute streams, so one chunk's last wave overlaps the
    // next chunk's first (they touch disjoint walkers; shared histograms use atomics).  With
    // three or more chunks the first and the last are a third of the others: only the first
    // chunk's copy in and the last chunk's copy out are not hidden behind sweeps.
    cudaStream_t comp[2] = {h->stream, h->s_comp2};
    const long long wsum = n_chunks >= 3 ? 3ll * (n_chunks - 2) + 2 : n_chunks;
    auto cut = [&](int k) -> int {  // first CTA of chunk k (k = n_chunks: the grid)
        long long wk = n_chunks >= 3 ? (k == 0 ? 0 : 1 + 3ll * (std::min(k, n_chunks - 1) - 1) + (k == n_chunks ? 1 : 0))
                                     : k;
        return (int)((long long)h->grid * wk / wsum);
    };
    for (int k = 0; k < n_chunks; k++) {
        const int cta0 = cut(k);
        const int cta1 = cut(k + 1);
        const size_t w0 = (size_t)cta0 * h->wpb;
        const size_t w1 = std::min((size_t)cta1 * h->wpb, (size_t)c.n_walkers);
        if (cta1 <= cta0 || w1 <= w0) continue;
        cudaEvent_t e_in = h->ev_chunk[2 * k], e_done = h->ev_chunk[2 * k + 1];
        CUDA_TRY(h, cudaMemcpyAsync((char *)h->d_paths + w0 * bpw, (const char *)paths_in + w0 * bpw, (w1 - w0) * bpw,
                                    cudaMemcpyHostToDevice, h->s_in), FS_ERR_CUDA);
        CUDA_TRY(h, cudaEventRecord(e_in, h->s_in), FS_ERR_CUDA);
        cudaStream_t cs = comp[k & 1];
        CUDA_TRY(h, cudaStreamWaitEvent(cs, e_in, 0), FS_ERR_CUDA);
        a.block_offset = cta0;
        for (int i = 0; i < n_launches; i++) {
            a.step_base = h->steps_done + per_launch * (unsigned long long)i;
            if (h->d_snap)
                CUDA_TRY(h, cudaMemcpyAsync(h->d_snap, h->d_seeds, (h->n_threads + 1) * 16, cudaMemcpyDeviceToDevice,
                                            cs), FS_ERR_CUDA);
            CUDA_TRY(h, cudaLaunchKernel((const void *)h->k_metro, dim3(cta1 - cta0), dim3(h->block), args, h->smem,
                                         cs), FS_ERR_LAUNCH);
        }
        CUDA_TRY(h, cudaEventRecord(e_done, cs), FS_ERR_CUDA);
        CUDA_TRY(h, cudaStreamWaitEvent(h->s_out, e_done, 0), FS_ERR_CUDA);
        CUDA_TRY(h, cudaMemcpyAsync((char *)paths_out + w0 * bpw, (const char *)h->d_paths + w0 * bpw, (w1 - w0) * bpw,
                                    cudaMemcpyDeviceToHost, h->s_out), FS_ERR_CUDA);
    }
    h->steps_done += per_launch * (unsigned long long)n_launches;
    // the handle's stream (fs_sync, the getters) waits for the second compute stream and
    // the last copy out
    cudaEvent_t e_end = h->ev_chunk[2 * n_chunks], e_c2 = h->ev_chunk[2 * n_chunks + 1];
    CUDA_TRY(h, cudaEventRecord(e_end, h->s_out), FS_ERR_CUDA);
    CUDA_TRY(h, cudaEventRecord(e_c2, h->s_comp2), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamWaitEvent(h->stream, e_end, 0), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamWaitEvent(h->stream, e_c2, 0), FS_ERR_CUDA);
    CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream), FS_ERR_CUDA);
    h->timed = true;
    h->status_pending = true;
    return FS_OK;
}

extern "C" int fs_get_last_chunks(const fs_handle *h, int32_t *chunks)
{
    if (!h || !chunks) return FS_ERR_CONFIG;
    *chunks = h->last_chunks;
    return FS_OK;
}

extern "C" int fs_pin_host(void *ptr, size_t bytes)
{
    cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, FS_ERR_CUDA, "cudaHostRegister: %s", cudaGetErrorString(e));
    }
    return FS_OK;
}

extern "C" int fs_unpin_host(void *ptr)
{
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, FS_ERR_CUDA, "cudaHostUnregister: %s", cudaGetErrorString(e));
    }
    return FS_OK;
}

static void fill_args(fs_handle *h, FsArgsHost &a)
{
    const fs_config &c = h->cfg;
    a.paths = h->d_paths;
    a.accepts = h->d_accepts;
    a.seeds = h->d_seeds;
    a.seed_snap = h->d_snap;
    a.walker_seeds = h->d_wseeds;
    a.rtab = h->d_rtab;
    a.gtab = h->d_gtab;
    a.op_means = h->d_ops;
    a.cor_means = h->d_cor;
    a.bins = h->d_bins;
    a.hist = h->d_hist;
    a.status = h->d_status;
    a.opnorm = 1.0 / ((double)c.operator_runs * c.n_slices * c.n_walkers / (double)h->n_threads);
    a.mlp_frag = h->d_mlp_frag;
    a.mlp_bias = h->d_mlp_bias;
    a.mlp_inv_scale = (float)h->mlp_inv_scale;
    a.shift_old = h->d_shift_old;
    a.step_base = h->steps_done;
    a.block_offset = 0;
    a.vcache = h->d_vcache;
}

// After the stream has drained: the status word the sweeps since the last check wrote
// (fs_pimc.cuh, FS_STATUS_*), cleared once read.
static int check_status(fs_handle *h)
{
    if (!h->status_pending) return FS_OK;
    int st[2] = {0, 0};
    CUDA_TRY(h, cudaMemcpyAsync(st, h->d_status, sizeof st, cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    h->status_pending = false;
    if (!st[0]) return FS_OK;
    CUDA_TRY(h, cudaMemsetAsync(h->d_status, 0, sizeof st, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return fail(h, FS_ERR_NUMERIC,
                "walker %d: a path value is not finite (NaN or infinity) after the sweep; the paths and the "
                "operator, correlator and histogram sums of this run are not usable", st[1] - 1);
}

extern "C" int fs_sync(fs_handle *h)
{
    if (!h) return FS_ERR_CONFIG;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return check_status(h);
}

// host watchdog: poll the stream instead of blocking forever (kernel.py:499-506 analogue)
extern "C" int fs_sync_timeout(fs_handle *h, double seconds)
{
    if (!h) return FS_ERR_CONFIG;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(h->stream);
        if (e == cudaSuccess) return check_status(h);
        if (e != cudaErrorNotReady) return fail(h, FS_ERR_LAUNCH, "stream error: %s", cudaGetErrorString(e));
        double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > seconds)
            return fail(h, FS_ERR_TIMEOUT, "work still running after %.3f s (limit %.3f s)", el, seconds);
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

extern "C" int fs_get_run_time(fs_handle *h, double *seconds)
{
    if (!h || !seconds) return FS_ERR_CONFIG;
    if (!h->timed) return fail(h, FS_ERR_STATE, "no run yet");
    CUDA_TRY(h, cudaEventSynchronize(h->ev1), FS_ERR_LAUNCH);
    float ms = 0.f;
    CUDA_TRY(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1), FS_ERR_CUDA);
    *seconds = ms * 1e-3;
    return FS_OK;
}

template <class T>
static void widen(const std::vector<unsigned char> &raw, double *out, size_t n)
{
    const T *p = (const T *)raw.data();
    for (size_t i = 0; i < n; i++) out[i] = (double)p[i];
}

extern "C" int fs_get_operators(fs_handle *h, double *out, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    if (n != h->n_ops_elems) return fail(h, FS_ERR_IO, "expected %zu operator values", h->n_ops_elems);
    std::vector<unsigned char> raw(n * h->op_elem + 1);
    int rc = copy_out(h, raw.data(), h->d_ops, n * h->op_elem, n * h->op_elem);
    if (rc) return rc;
    if (h->op_elem == 4) widen<float>(raw, out, n);
    else widen<double>(raw, out, n);
    return FS_OK;
}

// per-walker operator means: the mean over the walker's own threads of their per-thread
// means (thread ids as in the sweep, kernel.c:539-541), FP64, out[op][walker]
template <class T>
__global__ void fs_walker_ops_kernel(const T *ops, int n_walkers, int tpw, int wpg, int nwg, int nops, int parallel,
                                     double *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_walkers * nops) return;
    const int op = i / n_walkers, w = i - op * n_walkers;
    double s = 0.0;
    for (int t = 0; t < tpw; t++) {
        const long long tid = parallel ? (long long)(w / wpg) * tpw + t + (long long)(w % wpg) * nwg * tpw : w;
        s += (double)ops[tid * nops + op];
    }
    out[(size_t)op * n_walkers + w] = s / tpw;
}

extern "C" int fs_get_walker_operators(fs_handle *h, double *out, size_t n)
{
    if (!h || !out) return FS_ERR_CONFIG;
    const fs_config &c = h->cfg;
    const int nops = (int)h->ops.size();
    if (n != (size_t)nops * c.n_walkers) return fail(h, FS_ERR_IO, "expected %zu values", (size_t)nops * c.n_walkers);
    if (c.accum == 3) return fail(h, FS_ERR_STATE, "study accumulation keeps three columns: use fs_get_operators");
    if (nops == 0) return FS_OK;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    if (!h->d_wops) CUDA_TRY(h, cudaMalloc((void **)&h->d_wops, n * sizeof(double)), FS_ERR_OOM);
    const unsigned grid = (unsigned)((n + 255) / 256);
    const int par = c.enable_parallelize_path ? 1 : 0;
    const int nwg = c.n_walkers / std::max(1, c.walkers_per_group);
    if (h->op_elem == 8)
        fs_walker_ops_kernel<double><<<grid, 256, 0, h->stream>>>((const double *)h->d_ops, c.n_walkers, h->tpw,
                                                                  c.walkers_per_group, nwg, nops, par, h->d_wops);
    else
        fs_walker_ops_kernel<float><<<grid, 256, 0, h->stream>>>((const float *)h->d_ops, c.n_walkers, h->tpw,
                                                                 c.walkers_per_group, nwg, nops, par, h->d_wops);
    CUDA_TRY(h, cudaGetLastError(), FS_ERR_LAUNCH);
    CUDA_TRY(h, cudaMemcpyAsync(out, h->d_wops, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

extern "C" int fs_get_correlator(fs_handle *h, double *out, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    if (n != h->n_cor_elems) return fail(h, FS_ERR_IO, "expected %zu correlator values", h->n_cor_elems);
    const size_t bytes = h->n_cor_lags * h->cor_elem;
    std::vector<unsigned char> raw(bytes + 1);
    int rc = copy_out(h, raw.data(), h->d_cor, bytes, bytes);
    if (rc) return rc;
    if (h->cor_elem == 24) {
        for (size_t i = 0; i < h->n_cor_lags; i++) {
            FsCorStudyHost v;
            memcpy(&v, raw.data() + i * 24, 24);
            out[4 * i + 0] = v.f;
            out[4 * i + 1] = v.ks;
            out[4 * i + 2] = v.kc;
            out[4 * i + 3] = v.d;
        }
    } else if (h->cor_elem == 4) {
        widen<float>(raw, out, n);
    } else {
        widen<double>(raw, out, n);
    }
    return FS_OK;
}

extern "C" int fs_get_accepts(fs_handle *h, uint32_t *out, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, out, h->d_accepts, n * 4, (size_t)h->n_threads * 4);
}
extern "C" int fs_get_bins(fs_handle *h, uint32_t *out, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, out, h->d_bins, n * 4, h->n_bins * 4);
}
extern "C" int fs_get_histogram(fs_handle *h, uint64_t *out, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_out(h, out, h->d_hist, n * 8, h->n_hist * 8);
}
template <class T>
static int set_widened(fs_handle *h, void *dst, const double *in, size_t n)
{
    std::vector<T> tmp(n + 1);
    for (size_t i = 0; i < n; i++) tmp[i] = (T)in[i];
    return copy_in(h, dst, tmp.data(), n * sizeof(T), n * sizeof(T));
}

extern "C" int fs_set_correlator(fs_handle *h, const double *in, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    if (n != h->n_cor_elems) return fail(h, FS_ERR_IO, "expected %zu correlator values", h->n_cor_elems);
    if (n == 0) return FS_OK;
    if (h->cor_elem == 24) {
        std::vector<FsCorStudyHost> tmp(h->n_cor_lags + 1);
        for (size_t i = 0; i < h->n_cor_lags; i++)
            tmp[i] = FsCorStudyHost{in[4 * i + 3], (float)in[4 * i + 0], (float)in[4 * i + 1], (float)in[4 * i + 2], 0.f};
        return copy_in(h, h->d_cor, tmp.data(), h->n_cor_lags * 24, h->n_cor_lags * 24);
    }
    return h->cor_elem == 4 ? set_widened<float>(h, h->d_cor, in, n) : set_widened<double>(h, h->d_cor, in, n);
}

// ---- correlator moments over a walker range, on the device ----
// Block b reduces walkers [w0 + b*chunk, ...) for every lag (threads stride the lags, so
// a warp reads consecutive lags of one walker) and adds its partial sums atomically.
template <int KIND>  // 0: float, 1: double, 2: study struct (3 columns)
__global__ void fs_cor_moments_kernel(const unsigned char *cor, size_t lags, long long w0, long long w1,
                                      long long chunk, double *sum, double *sq)
{
    constexpr int NC = KIND == 2 ? 3 : 1;
    const long long wb = w0 + (long long)blockIdx.x * chunk;
    const long long we = wb + chunk < w1 ? wb + chunk : w1;
    for (size_t l = threadIdx.x; l < lags; l += blockDim.x) {
        double s[NC], q[NC];
#pragma unroll
        for (int k = 0; k < NC; k++) s[k] = q[k] = 0.0;
        for (long long w = wb; w < we; w++) {
            const size_t i = (size_t)w * lags + l;
            double v[NC];
            if (KIND == 0) {
                v[0] = (double)((const float *)cor)[i];
            } else if (KIND == 1) {
                v[0] = ((const double *)cor)[i];
            } else {
                const unsigned char *e = cor + i * 24;
                v[0] = (double)*(const float *)(e + 8);
                v[NC > 1 ? 1 : 0] = (double)*(const float *)(e + 12);
                v[NC > 2 ? 2 : 0] = *(const double *)e;
            }
#pragma unroll
            for (int k = 0; k < NC; k++) {
                s[k] += v[k];
                q[k] += v[k] * v[k];
            }
        }
#pragma unroll
        for (int k = 0; k < NC; k++) {
            atomicAdd(sum + l * NC + k, s[k]);
            atomicAdd(sq + l * NC + k, q[k]);
        }
    }
}

extern "C" int fs_reduce_correlator(fs_handle *h, int64_t walker_begin, int64_t walker_end, double *sum,
                                    double *sumsq, size_t n)
{
    if (!h || !sum || !sumsq) return FS_ERR_CONFIG;
    const size_t W = (size_t)h->cfg.n_walkers;
    const size_t lags = h->cors.size() * (size_t)(h->cfg.n_slices / 2);
    const int ncol = h->cor_elem == 24 ? 3 : 1;
    if (lags == 0) return fail(h, FS_ERR_STATE, "no correlators");
    if (n != lags * ncol) return fail(h, FS_ERR_IO, "expected %zu values", lags * ncol);
    if (walker_begin < 0 || walker_end > (int64_t)W || walker_begin >= walker_end)
        return fail(h, FS_ERR_IO, "walker range [%lld, %lld) outside [0, %zu)", (long long)walker_begin,
                    (long long)walker_end, W);
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    if (!h->d_red) CUDA_TRY(h, cudaMalloc((void **)&h->d_red, 2 * lags * 3 * sizeof(double)), FS_ERR_OOM);
    CUDA_TRY(h, cudaMemsetAsync(h->d_red, 0, 2 * n * sizeof(double), h->stream), FS_ERR_CUDA);
    const long long nw = walker_end - walker_begin;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, h->device);
    const long long blocks = std::min<long long>(nw, (long long)sms * 8);
    const long long chunk = (nw + blocks - 1) / blocks;
    const unsigned grid = (unsigned)((nw + chunk - 1) / chunk);
    const unsigned char *c = (const unsigned char *)h->d_cor;
    double *s = h->d_red, *q = h->d_red + n;
    if (h->cor_elem == 24)
        fs_cor_moments_kernel<2><<<grid, 256, 0, h->stream>>>(c, lags, walker_begin, walker_end, chunk, s, q);
    else if (h->cor_elem == 8)
        fs_cor_moments_kernel<1><<<grid, 256, 0, h->stream>>>(c, lags, walker_begin, walker_end, chunk, s, q);
    else
        fs_cor_moments_kernel<0><<<grid, 256, 0, h->stream>>>(c, lags, walker_begin, walker_end, chunk, s, q);
    CUDA_TRY(h, cudaGetLastError(), FS_ERR_LAUNCH);
    CUDA_TRY(h, cudaMemcpyAsync(sum, s, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaMemcpyAsync(sumsq, q, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

extern "C" int fs_set_paths_tiled(fs_handle *h, const void *host, size_t n_template)
{
    if (!h || !host) return FS_ERR_CONFIG;
    const size_t W = (size_t)h->cfg.n_walkers;
    if (n_template == 0 || n_template > W)
        return fail(h, FS_ERR_IO, "template walker count %zu outside [1, %zu]", n_template, W);
    const size_t wb = (size_t)h->cfg.dof * h->cfg.n_slices * h->ft;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    CUDA_TRY(h, cudaMemcpyAsync(h->d_paths, host, n_template * wb, cudaMemcpyHostToDevice, h->stream), FS_ERR_CUDA);
    // doubling copies: walkers [0, k) -> [k, 2k) keep w % n_template because k is a
    // multiple of n_template
    size_t k = n_template;
    while (k < W) {
        const size_t m = std::min(k, W - k);
        CUDA_TRY(h, cudaMemcpyAsync((char *)h->d_paths + k * wb, h->d_paths, m * wb, cudaMemcpyDeviceToDevice,
                                    h->stream), FS_ERR_CUDA);
        k += m;
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}
extern "C" int fs_set_bins(fs_handle *h, const uint32_t *in, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_in(h, h->d_bins, in, n * 4, h->n_bins * 4);
}
extern "C" int fs_set_histogram(fs_handle *h, const uint64_t *in, size_t n)
{
    if (!h) return FS_ERR_CONFIG;
    return copy_in(h, h->d_hist, in, n * 8, h->n_hist * 8);
}

extern "C" int fs_zero_accumulators(fs_handle *h)
{
    if (!h) return FS_ERR_CONFIG;
    CUDA_TRY(h, cudaSetDevice(h->device), FS_ERR_CUDA);
    if (h->n_cor_lags) CUDA_TRY(h, cudaMemsetAsync(h->d_cor, 0, h->n_cor_lags * h->cor_elem, h->stream), FS_ERR_CUDA);
    if (h->n_bins) CUDA_TRY(h, cudaMemsetAsync(h->d_bins, 0, h->n_bins * 4, h->stream), FS_ERR_CUDA);
    if (h->n_hist) CUDA_TRY(h, cudaMemsetAsync(h->d_hist, 0, h->n_hist * 8, h->stream), FS_ERR_CUDA);
    CUDA_TRY(h, cudaStreamSynchronize(h->stream), FS_ERR_LAUNCH);
    return FS_OK;
}

// ------------------------------------------------------------------ RNG stream modules
static std::mutex g_rng_mu;
static std::unordered_map<int, cudaLibrary_t> g_rng_libs;  // per (device, lux)

static int rng_module(int lux, cudaLibrary_t *lib)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return fail(nullptr, FS_ERR_CUDA, "no CUDA device");
    const int key = dev * 4096 + lux;
    std::lock_guard<std::mutex> lk(g_rng_mu);
    auto it = g_rng_libs.find(key);
    if (it != g_rng_libs.end()) {
        *lib = it->second;
        return FS_OK;
    }
    std::ostringstream o;
    o << gen_prelude(false) << "#define FS_NSKIP " << nskip_for(lux) << "\n#define FS_RNG_ONLY 1\n"
      << "#define FS_N 2\n#define FS_S 0\n#define FS_SEG 1\n#define FS_TPW 1\n#define FS_WPB 1\n"
         "#define FS_NWALKERS 1\n#define FS_WPG 1\n#define FS_NWG 1\n#define FS_PARALLEL 0\n#define FS_MINB 0\n"
         "#define FS_WSTRIDE 16\n#define FS_LEARNED 0\n"
         "#define FS_RANLUX 0\n#define FS_COMPAT 0\n#define FS_ACCUM 1\n#define FS_FAST 0\n"
         "#define FS_NOPS 0\n#define FS_NCOR 0\n#define FS_OPRUNS 1\n#define FS_MSTEPS 1\n"
         "#define FS_EPS 1.0f\n#define FS_OPNORM 1.0f\n#define FS_BINS 0\n#define FS_NHIST 0\n"
         "#define FS_HBINS 0\n#define FS_RIM 4.294967296E+09f\n#define FS_DOF 1\n"
      << kRngSrc << "\n#define FS_ARGS_AT(P, i) (P)[(i)]\n__constant__ FT fs_sigma[1] = {0.0f};\n"
      << "__device__ FT fs_pot(FT x1) { return x1; }\n" << kPimcSrc;
    fs_handle tmp;
    std::string cubin, log;
    int rc = compile_module(&tmp, o.str(), false, &cubin, &log);
    if (rc) return fail(nullptr, rc, "%s", tmp.err.c_str());
    cudaError_t e = cudaLibraryLoadData(lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) return fail(nullptr, FS_ERR_CUDA, "cudaLibraryLoadData: %s", cudaGetErrorString(e));
    g_rng_libs[key] = *lib;
    return FS_OK;
}

#define G_TRY(call)                                                                     \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            fail(nullptr, FS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));         \
            goto done;                                                                  \
        }                                                                               \
    } while (0)

extern "C" int fs_rng_ranlux_stream(int32_t lux, const uint64_t *xs, int32_t n, int32_t calls, float *out,
                                    uint32_t *states)
{
    int ns = nskip_for(lux);
    if (lux < 0 || (lux > 4 && lux < 24) || ns % 4 || (ns && ns < 24) || n < 1 || calls < 0)
        return fail(nullptr, FS_ERR_CONFIG, "bad RANLUX stream request");
    cudaLibrary_t lib;
    int rc = rng_module(lux, &lib);
    if (rc) return rc;
    cudaKernel_t k;
    void *dx = nullptr, *dout = nullptr, *dst = nullptr;
    rc = FS_ERR_CUDA;
    G_TRY(cudaLibraryGetKernel(&k, lib, "fs_ranlux_dump"));
    G_TRY(cudaMalloc(&dx, (size_t)n * 8));
    G_TRY(cudaMalloc(&dout, (size_t)n * calls * 16 + 16));
    G_TRY(cudaMalloc(&dst, (size_t)n * 112));
    G_TRY(cudaMemcpy(dx, xs, (size_t)n * 8, cudaMemcpyHostToDevice));
    {
        void *args[] = {&dx, &n, &calls, &dout, &dst};
        G_TRY(cudaLaunchKernel((const void *)k, dim3((n + 63) / 64), dim3(64), args, 0, 0));
    }
    G_TRY(cudaDeviceSynchronize());
    G_TRY(cudaMemcpy(out, dout, (size_t)n * calls * 16, cudaMemcpyDeviceToHost));
    if (states) G_TRY(cudaMemcpy(states, dst, (size_t)n * 112, cudaMemcpyDeviceToHost));
    rc = FS_OK;
done:
    if (dx) cudaFree(dx);
    if (dout) cudaFree(dout);
    if (dst) cudaFree(dst);
    return rc;
}

extern "C" int fs_rng_ranlux_stream64(int32_t lux, const uint64_t *xs, int32_t n, int32_t calls, double *out)
{
    int ns = nskip_for(lux);
    if (lux < 0 || (lux > 4 && lux < 24) || ns % 4 || (ns && ns < 24) || n < 1 || calls < 0)
        return fail(nullptr, FS_ERR_CONFIG, "bad RANLUX stream request");
    cudaLibrary_t lib;
    int rc = rng_module(lux, &lib);
    if (rc) return rc;
    cudaKernel_t k;
    void *dx = nullptr, *dout = nullptr;
    rc = FS_ERR_CUDA;
    G_TRY(cudaLibraryGetKernel(&k, lib, "fs_ranlux_dump64"));
    G_TRY(cudaMalloc(&dx, (size_t)n * 8));
    G_TRY(cudaMalloc(&dout, (size_t)n * calls * 32 + 32));
    G_TRY(cudaMemcpy(dx, xs, (size_t)n * 8, cudaMemcpyHostToDevice));
    {
        void *args[] = {&dx, &n, &calls, &dout};
        G_TRY(cudaLaunchKernel((const void *)k, dim3((n + 63) / 64), dim3(64), args, 0, 0));
    }
    G_TRY(cudaDeviceSynchronize());
    G_TRY(cudaMemcpy(out, dout, (size_t)n * calls * 32, cudaMemcpyDeviceToHost));
    rc = FS_OK;
done:
    if (dx) cudaFree(dx);
    if (dout) cudaFree(dout);
    return rc;
}

extern "C" int fs_rng_xorshift_stream(uint32_t *states, int32_t n, int32_t draws, uint32_t *out, float *fout)
{
    if (n < 1 || draws < 0) return fail(nullptr, FS_ERR_CONFIG, "bad xorshift stream request");
    cudaLibrary_t lib;
    int rc = rng_module(0, &lib);
    if (rc) return rc;
    cudaKernel_t k;
    void *ds = nullptr, *dout = nullptr, *dfo = nullptr;
    rc = FS_ERR_CUDA;
    G_TRY(cudaLibraryGetKernel(&k, lib, "fs_xorshift_dump"));
    G_TRY(cudaMalloc(&ds, (size_t)n * 16));
    G_TRY(cudaMalloc(&dout, (size_t)n * draws * 4 + 4));
    G_TRY(cudaMalloc(&dfo, (size_t)n * draws * 4 + 4));
    G_TRY(cudaMemcpy(ds, states, (size_t)n * 16, cudaMemcpyHostToDevice));
    {
        void *args[] = {&ds, &n, &draws, &dout, &dfo};
        G_TRY(cudaLaunchKernel((const void *)k, dim3((n + 63) / 64), dim3(64), args, 0, 0));
    }
    G_TRY(cudaDeviceSynchronize());
    G_TRY(cudaMemcpy(out, dout, (size_t)n * draws * 4, cudaMemcpyDeviceToHost));
    G_TRY(cudaMemcpy(fout, dfo, (size_t)n * draws * 4, cudaMemcpyDeviceToHost));
    G_TRY(cudaMemcpy(states, ds, (size_t)n * 16, cudaMemcpyDeviceToHost));
    rc = FS_OK;
done:
    if (ds) cudaFree(ds);
    if (dout) cudaFree(dout);
    if (dfo) cudaFree(dfo);
    return rc;
}

// Host side of the dense passes (the kernels are in dense_pass.cuh, one
// translation unit per element type and launch configuration): launch with
// the configuration the autotuner chose, grid sizes, the FP32 split of the
// pass vectors, and the autotuner's table of choices with its cache file.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "internal.h"

namespace regot {

thread_local long long* g_launch_counter = nullptr;

int device_sm_count() {
    int dev = 0, count = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    static std::atomic<int> cache[64] = {};
    if (dev < 64) {
        const int c = cache[dev].load(std::memory_order_relaxed);
        if (c) return c;
    }
    if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        count <= 0)
        count = 1;
    if (dev < 64) cache[dev].store(count, std::memory_order_relaxed);
    return count;
}

namespace {
std::atomic<long long> g_wait_limit{kDefaultWaitSpins};

__device__ __forceinline__ void split(double v, double g, double inv_g, float& hi, float& lo) {
    if (!isfinite(v)) {
        hi = (float)v;
        lo = 0.f;
        return;
    }
    const double h = rint(v * inv_g) * g;
    hi = (float)h;
    lo = (float)(v - h);
}

// FP32 copies of the per-row / per-column vectors of a mixed pass; the duals
// are split on the common grid G = 2^(floor(log2 bound) - 21).
__global__ void k_split(const PassParams p, float4* rs, float4* cs, float* cds) {
    double g = 1.0, inv_g = 1.0;
    if (p.grid) {
        const double mx = *p.grid;
        if (mx > 0.0 && isfinite(mx)) {
            const int e = ilogb(mx) - 21;
            g = ldexp(1.0, e);
            inv_g = ldexp(1.0, -e);
        }
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < p.n) {
        float hi = 0.f, lo = 0.f;
        if (p.ra) split(p.ra[t], g, inv_g, hi, lo);
        rs[t] = make_float4(hi, lo, p.rx ? (float)p.rx[t] : 0.f, p.rd ? (float)p.rd[t] : 0.f);
    } else if (t < p.n + p.m) {
        const int j = t - p.n;
        float hi = 0.f, lo = 0.f;
        if (p.cb) split(p.cb[j], g, inv_g, hi, lo);
        cs[j] = make_float4(hi, lo, p.cx ? (float)p.cx[j] : 0.f, p.cx2 ? (float)p.cx2[j] : 0.f);
        if (cds) cds[j] = p.cd ? (float)p.cd[j] : 0.f;
    }
}


// ---------------------------------------------------------- autotuner --
// Choices keyed by (device name, precision, pass, size class): the size
// class of an n x m pass is floor(log2(n m)). A lookup without an entry for
// its class takes the nearest tuned class of the same pass within two
// classes, else configuration 0.
struct TuneKey {
    std::string device;
    int mixed, op, bucket;
    bool operator<(const TuneKey& o) const {
        return std::tie(device, mixed, op, bucket) < std::tie(o.device, o.mixed, o.op, o.bucket);
    }
};
struct TuneVal {
    int cfg;
    double us[kPassConfigs];
};
std::mutex g_tune_mutex;
std::map<TuneKey, TuneVal> g_tune;
bool g_tune_loaded = false;
std::atomic<int> g_force_cfg{-1};

std::string current_device_name() {
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess)
        return "unknown";
    std::string name = prop.name;
    for (char& c : name)
        if (c == '\t' || c == '\n') c = ' ';
    return name + " sm" + std::to_string(prop.multiProcessorCount);
}

std::string default_cache_path() {
    if (const char* p = std::getenv("REGOT_GB300_AUTOTUNE")) return p;
    if (const char* h = std::getenv("HOME")) return std::string(h) + "/.cache/regot_gb300_autotune.tsv";
    return "";
}

// Lines: device <TAB> precision (fp64 | mixed) <TAB> pass <TAB> size class
// <TAB> configuration <TAB> microseconds of each configuration.
int load_locked(const std::string& path) {
    FILE* f = path.empty() ? nullptr : std::fopen(path.c_str(), "r");
    if (!f) return 0;
    char line[512];
    int count = 0;
    while (std::fgets(line, sizeof(line), f)) {
        char* fields[5 + kPassConfigs];
        int nf = 0;
        char* save = nullptr;
        for (char* tok = strtok_r(line, "\t\n", &save); tok && nf < 5 + kPassConfigs;
             tok = strtok_r(nullptr, "\t\n", &save))
            fields[nf++] = tok;
        if (nf < 5) continue;
        TuneKey k{fields[0], std::strcmp(fields[1], "mixed") == 0 ? 1 : 0, std::atoi(fields[2]),
                  std::atoi(fields[3])};
        TuneVal v{std::atoi(fields[4]), {}};
        if (v.cfg < 0 || v.cfg >= kPassConfigs || k.op < 0 || k.op >= OP_COUNT) continue;
        for (int c = 0; c < kPassConfigs; ++c) v.us[c] = 5 + c < nf ? std::atof(fields[5 + c]) : 0.0;
        g_tune[k] = v;
        ++count;
    }
    std::fclose(f);
    return count;
}

void ensure_loaded() {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    if (!g_tune_loaded) {
        g_tune_loaded = true;
        load_locked(default_cache_path());
    }
}

int size_class(int n, int m) { return (int)std::floor(std::log2((double)n * (double)m)); }
}  // namespace

long long wait_limit() { return g_wait_limit.load(std::memory_order_relaxed); }
long long set_wait_limit(long long spins) {
    return g_wait_limit.exchange(spins < 0 ? kDefaultWaitSpins : spins);
}

int force_pass_config(int cfg) {
    return g_force_cfg.exchange(cfg >= 0 && cfg < kPassConfigs ? cfg : -1);
}

int pass_config(int op, bool mixed, int n, int m) {
    const int forced = g_force_cfg.load(std::memory_order_relaxed);
    if (forced >= 0) return forced;
    ensure_loaded();
    static thread_local std::string dev_name;
    static thread_local int dev_of_name = -1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (dev != dev_of_name) {
        dev_name = current_device_name();
        dev_of_name = dev;
    }
    const int b = size_class(n, m);
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    for (int d = 0; d <= 2; ++d)
        for (int sgn = -1; sgn <= 1; sgn += 2) {
            auto it = g_tune.find(TuneKey{dev_name, mixed ? 1 : 0, op, b + sgn * d});
            if (it != g_tune.end()) return it->second.cfg;
            if (d == 0) break;
        }
    return 0;
}

void record_tuning(int op, bool mixed, int n, int m, int cfg, const double* us) {
    ensure_loaded();
    TuneVal v{cfg, {}};
    for (int c = 0; c < kPassConfigs; ++c) v.us[c] = us[c];
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune[TuneKey{current_device_name(), mixed ? 1 : 0, op, size_class(n, m)}] = v;
}

int save_tuning(const char* path) {
    const std::string p = path && *path ? std::string(path) : default_cache_path();
    if (p.empty()) return -1;
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    FILE* f = std::fopen(p.c_str(), "w");
    if (!f) return -1;
    for (const auto& kv : g_tune) {
        std::fprintf(f, "%s\t%s\t%d\t%d\t%d", kv.first.device.c_str(),
                     kv.first.mixed ? "mixed" : "fp64", kv.first.op, kv.first.bucket, kv.second.cfg);
        for (int c = 0; c < kPassConfigs; ++c) std::fprintf(f, "\t%.3f", kv.second.us[c]);
        std::fprintf(f, "\n");
    }
    std::fclose(f);
    return (int)g_tune.size();
}

int load_tuning(const char* path) {
    const std::string p = path && *path ? std::string(path) : default_cache_path();
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_loaded = true;
    return load_locked(p);
}

void clear_tuning() {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune.clear();
    g_tune_loaded = true;
}

std::string tuning_entries() {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    std::string out;
    char buf[128];
    for (const auto& kv : g_tune) {
        std::snprintf(buf, sizeof(buf), "\t%s\t%d\t%d\t%d", kv.first.mixed ? "mixed" : "fp64",
                      kv.first.op, kv.first.bucket, kv.second.cfg);
        out += kv.first.device + buf;
        for (int c = 0; c < kPassConfigs; ++c) {
            std::snprintf(buf, sizeof(buf), "\t%.3f", kv.second.us[c]);
            out += buf;
        }
        out += "\n";
    }
    return out;
}

// ------------------------------------------------------------ launches --
namespace {
int occupancy(int op, bool mixed, int cfg) {
    int dev = 0;
    REGOT_CUDA(cudaGetDevice(&dev));
    static std::atomic<int> cache[64][2][kPassConfigs][OP_COUNT] = {};
    const bool ok = dev < 64 && op >= 0 && op < OP_COUNT;
    int occ = ok ? cache[dev][mixed][cfg][op].load(std::memory_order_relaxed) : 0;
    if (!occ) {
        if (cfg == 0) occ = mixed ? occupancy_cfg<float, 0>(op) : occupancy_cfg<double, 0>(op);
        else occ = mixed ? occupancy_cfg<float, 1>(op) : occupancy_cfg<double, 1>(op);
        if (ok) cache[dev][mixed][cfg][op].store(occ, std::memory_order_relaxed);
    }
    return occ;
}

int blocks_for(int op, bool mixed, int n, int m, int cfg) {
    const PassShape s = mixed ? pass_shape<float>(n, m) : pass_shape<double>(n, m);
    const int cap = device_sm_count() * occupancy(op, mixed, cfg);
    return s.ntiles < cap ? s.ntiles : cap;
}
}  // namespace

template <typename TM>
void launch_pass(int op, const PassParams& p, cudaStream_t st) {
    if (p.n <= 0 || p.m <= 0) return;
    PassParams q = p;
    q.kexp_f = (float)(1.4426950408889634 / p.reg);
    q.inv_kexp_f = 1.0f / q.kexp_f;
    q.inv_reg_f = (float)(1.0 / p.reg);
    q.kexp_d = 1.0 / p.reg;
    q.inv_reg_d = 1.0 / p.reg;
    q.wait_limit = wait_limit();
    constexpr bool mixed = std::is_same<TM, float>::value;
    const int cfg = pass_config(op, mixed, p.n, p.m);
    const int blocks = blocks_for(op, mixed, p.n, p.m, cfg);
    if (cfg == 0) launch_pass_cfg<TM, 0>(op, q, st, blocks);
    else launch_pass_cfg<TM, 1>(op, q, st, blocks);
}

int pass_blocks(int op, bool mixed, int n, int m) {
    return blocks_for(op, mixed, n, m, pass_config(op, mixed, n, m));
}

void launch_split(const PassParams& p, float4* rs, float4* cs, float* cds, cudaStream_t st) {
    k_split<<<cdiv(p.n + p.m, 64), 64, 0, st>>>(p, rs, cs, cds);
    REGOT_CHECK_LAUNCH();
    count_launch();
}

template void launch_pass<float>(int, const PassParams&, cudaStream_t);
template void launch_pass<double>(int, const PassParams&, cudaStream_t);

}  // namespace regot

// Internal declarations shared by the CUDA translation units of regot_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "regot_gb300.h"

namespace regot {

// ---------------------------------------------------------------- errors --
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

#define REGOT_CUDA(call)                                                                 \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            throw ::regot::Error(REGOT_ERR_CUDA, std::string(#call) + ": " +             \
                                                     cudaGetErrorString(e_));            \
    } while (0)

#define REGOT_CHECK_LAUNCH() REGOT_CUDA(cudaGetLastError())

inline void require(bool ok, const std::string& msg, int code = REGOT_ERR_INVALID_ARG) {
    if (!ok) throw Error(code, msg);
}

// Stream-ordered device allocation from the library's own memory pool of the
// current device. The pool keeps up to kPoolKeepBytes of freed memory mapped
// across synchronisations, so consecutive problems and solves reuse it
// instead of mapping fresh pages (the default pool returns everything at each
// synchronisation). Free with cudaFreeAsync.
constexpr unsigned long long kPoolKeepBytes = 4ULL << 30;
void* dev_alloc(size_t bytes, cudaStream_t st);

// ------------------------------------------------------------- geometry --
// Dense passes tile M (row-major, row stride ldm) into tiles of RB rows x
// CW columns. A CTA has 8 warps; each warp streams RB/8 consecutive rows of
// a tile and each lane owns LC / VW 16-byte vectors per row (16 FP32 or 8 FP64
// columns).
constexpr int kThreads = 256;            // 8 warps per CTA
constexpr int kWarps = kThreads / 32;
constexpr int kRB = 64;                  // rows per tile (8 per warp)

template <typename TM> struct Geo;
template <> struct Geo<float> {
    static constexpr int VW = 4;    // elements per 16-byte vector
    static constexpr int LC = 16;   // columns per lane
    static constexpr int CW = 512;  // columns per slab (one 2 KB row segment)
};
template <> struct Geo<double> {
    static constexpr int VW = 2;
    static constexpr int LC = 8;
    static constexpr int CW = 256;
};

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// Dense pass operations (see passes.cu for the element formulas).
enum PassOp : int {
    OP_E_ROW = 0,     // row sums of T
    OP_E_COL,         // column sums of T
    OP_E_ROWCOL,      // row and column sums of T
    OP_E_HVP,         // rows: sum_j T cx_j ; cols: sum_i T rx_i
    OP_E_LS,          // totals_k: sum T (e^w - 1 - w), w = s_k (rd_i + cd_j)/reg
    OP_E_PLAN,        // write T
    OP_E_ROWMAX,      // rows: max_j (cb_j - M_ij)
    OP_E_COLMAX,      // cols: max_i (ra_i - M_ij)
    OP_Q_GRAD,        // rows/cols: sum D ; total: sum D^2
    OP_Q_GRADMASK,    // + bitmask of C > 0, row/col counts
    OP_Q_OBJ,         // total: sum D^2
    OP_Q_P1,          // rows: sum D
    OP_Q_P2,          // cols: sum D rx_i
    OP_Q_P3,          // rows: sum D cx, sum D cx cx2, sum M cx2 ; totals
    OP_Q_PLAN,        // write D / reg
    OP_Q_COLROOT,     // cols: count and sum of y = M - ra below cb (FP64)
    OP_Q_GRADLS,      // at C + s w (w = rd_i + cd_j): rows/cols sum Dn; totals sum Dn^2,
                      // sum of 0.5 (Dn^2 - D^2) - s w D (second-order part of the change)
    OP_E_GRADLS,      // at the trial point (ra, cb), direction (rd, cd), step s: rows/cols
                      // sum T; total sum T e^(-s w) phi(s w), w = (rd_i + cd_j)/reg,
                      // phi(x) = e^x - 1 - x (change from the base point, minus s g'd, / reg)
    OP_E_AVG,         // averaged plan X <- (1 - s) X + s T (X = T when nsteps == 0), X at
                      // xavg (TM, row-major, stride m): rows/cols sum X; totals sum M X,
                      // sum X (1 - log X)
    OP_Q_ROWROOT,     // rows: count and sum of y = M - cb below ra (FP64), optimal_alpha
    OP_Q_AVG,         // averaged plan X <- steps[0] X + steps[1] D / reg (X = D / reg when
                      // nsteps == 0), X at xavg (TM, row-major, stride m): rows/cols sum X;
                      // totals sum M X, sum X^2
    OP_COUNT
};

// Parameters of one dense pass. Row vectors have n entries, column vectors
// m entries; all FP64 on the device.
struct PassParams {
    const void* M = nullptr;
    long long ldm = 0;
    int n = 0, m = 0;
    const double* ra = nullptr;  // row dual (alpha or anchor)
    const double* cb = nullptr;  // column dual (beta, full length m)
    const double* rx = nullptr;  // extra row weights
    const double* cx = nullptr;  // extra column weights
    const double* cx2 = nullptr;
    const double* rd = nullptr;  // line-search direction (rows)
    const double* cd = nullptr;  // line-search direction (cols)
    double steps[4] = {0, 0, 0, 0};
    int nsteps = 0;
    double reg = 1.0;
    const double* grid = nullptr;  // device scalar: bound on |ra|, |cb| (mixed hi/lo grid)
    // Mixed mode: FP32 copies prepared once per pass by the split kernel.
    const float4* rsplit = nullptr;  // per row: (hi, lo, rx, rd)
    const float4* csplit = nullptr;  // per column: (hi, lo, cx, cx2)
    const float* cdsplit = nullptr;  // per column: cd
    // Filled by launch_pass from reg.
    float kexp_f = 0.f, inv_kexp_f = 0.f, inv_reg_f = 0.f;
    double kexp_d = 0.0, inv_reg_d = 0.0;
    void* rowpart = nullptr;       // [NR][nslabs][n] (Acc)
    void* colpart = nullptr;       // [NC][nrb][m]   (Acc)
    double* totpart = nullptr;     // [NT][nblocks]
    uint32_t* bitmask = nullptr;   // [n][nslabs][LC]
    double* out = nullptr;         // plan output, row-major, stride m
    void* xavg = nullptr;          // averaged plan (OP_E_AVG, OP_Q_AVG), TM, row-major, stride m
    const int* done = nullptr;     // early-exit flag (device)
    int* err = nullptr;            // set to 1 if a bounded wait gave up (device)
    long long wait_limit = 0;      // polls before a wait gives up (filled by launch_pass)
};

// Polls (each suspended for up to 200 us) before a bounded wait on a copy
// barrier gives up: a few seconds at most.
constexpr long long kDefaultWaitSpins = 1LL << 14;
// Current limit of the dense passes' bounded waits, and a setter that
// returns the previous value (negative: back to kDefaultWaitSpins). A lower
// limit makes the waits give up early; the tests use it to exercise the
// timeout path without a fault.
long long wait_limit();
long long set_wait_limit(long long spins);

struct PassShape {
    int nslabs, nrb, ntiles;
    int nblocks;  // capacity for per-CTA totals (>= the grid of any dense pass)
};

// Launch configurations of the dense passes (dense_pass.cuh): CTAs per SM
// (the register budget: 128 registers a thread with 2, 255 with 1) and the
// depth of each warp's ring of row buffers. The autotuner (passes.cu)
// chooses one per (device, precision, pass, size class of n m).
template <int CFG> struct PassCfg;
template <> struct PassCfg<0> { static constexpr int kMinBlocks = 2, kStages = 4; };
template <> struct PassCfg<1> { static constexpr int kMinBlocks = 1, kStages = 8; };
constexpr int kPassConfigs = 2;
template <typename TM, int CFG>
void launch_pass_cfg(int op, const PassParams& p, cudaStream_t st, int blocks);
template <typename TM, int CFG>
int occupancy_cfg(int op);
// The configuration the passes use for (op, precision, n, m): a forced
// choice (tests, the tuner), else the tuned one, else 0.
int pass_config(int op, bool mixed, int n, int m);
// Force one configuration for every pass (-1: back to the tuned choices);
// returns the previous forced value.
int force_pass_config(int cfg);
// The autotuner's table (passes.cu): record a measured choice for the
// current device, save / load the cache file (NULL or "": the default path,
// $REGOT_GB300_AUTOTUNE or ~/.cache/regot_gb300_autotune.tsv), clear it,
// and list it (one line per entry, as in the file).
void record_tuning(int op, bool mixed, int n, int m, int cfg, const double* us);
int save_tuning(const char* path);
int load_tuning(const char* path);
void clear_tuning();
std::string tuning_entries();

constexpr int kMaxPassCtasPerSm = 4;
int device_sm_count();
// Grid of the persistent dense pass `op` (SMs x resident CTAs, at most the
// number of tiles); per-CTA totals of that pass have this many entries.
int pass_blocks(int op, bool mixed, int n, int m);

template <typename TM>
inline PassShape pass_shape(int n, int m) {
    PassShape s;
    s.nslabs = cdiv(m, Geo<TM>::CW);
    s.nrb = cdiv(n, kRB);
    s.ntiles = s.nslabs * s.nrb;
    const int cap = device_sm_count() * kMaxPassCtasPerSm;
    s.nblocks = s.ntiles < cap ? s.ntiles : cap;
    return s;
}

// Launch a dense pass (passes.cu).
template <typename TM>
void launch_pass(int op, const PassParams& p, cudaStream_t st);

// Mixed mode: fill p.rsplit / p.csplit / p.cdsplit (buffers of n, m, m
// entries) from the FP64 vectors of p, on the hi/lo grid of *p.grid.
void launch_split(const PassParams& p, float4* rs, float4* cs, float* cds, cudaStream_t st);

// Count of kernels launched (for gpu_launches accounting).
extern thread_local long long* g_launch_counter;
inline void count_launch(int k = 1) {
    if (g_launch_counter) *g_launch_counter += k;
}

}  // namespace regot

struct regot_ctx;
namespace regot {
// Page-locked staging block of the context, at least `bytes` long (grown on
// demand, freed with the context). A copy from the device to pageable memory
// is a blocking round trip per call; copies into this block are
// asynchronous, so several results come back behind one synchronisation.
void* ctx_stage(regot_ctx* ctx, size_t bytes);
// Blocking read of `bytes` (at most a few KB) from the device through the
// staging block.
void read_small(regot_ctx* ctx, void* dst, const void* src, size_t bytes, cudaStream_t st);
// Device address of host memory [p, p + bytes) when it lies inside one live
// block of regot_host_alloc (page-locked and mapped), else nullptr.
void* host_block_view(void* p, size_t bytes);
}  // namespace regot

// ---------------------------------------------------------- C-ABI objects --
struct regot_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    std::string last_error;
    long long launches = 0;
    void* stage = nullptr;  // page-locked staging for small device-to-host reads
    size_t stage_bytes = 0;
};

struct regot_dproblem {
    regot_ctx* ctx = nullptr;
    int n = 0, m = 0;
    long long ldm = 0;
    int prec = REGOT_PREC_MIXED;  // storage: FP64 or FP32
    void* M = nullptr;            // device, n x ldm
    double* a = nullptr;          // device
    double* b = nullptr;          // device
    double* loga = nullptr;       // device log(a), log(b): made by the first EROT solve
    double* logb = nullptr;
    std::vector<double> ha, hb;   // host copies
    double sum_a = 0.0;           // sum_i a_i
    double sum_bt = 0.0;          // sum_{j < m-1} b_j
};

// solver.cu — pfgb context, fused pass ops and the dynamics step.
//
// One dynamics step (reference sequence main_cuda.cu:28427-31623) becomes:
//   elastic  : [z eigen->R2C] [y] [x Green0 + strain] [y^-1]          (cold)
//              [x strain(u)] [y^-1]                                    (warm)
//              { [z C2R->h_ij->R2C] [y] [x Green(h)+resid+strain] [y^-1] } x iters
//              [z C2R -> eps + E0]
//   phi      : [z phi - L dt rhs -> R2C] [y] [x filter] [y^-1] [z C2R -> clamp]
//   eta (GP) : same as phi
//   Y        : [z mu -> R2C, sum DY] [y] [x grad] [y^-1]
//              [z C2R grad -> J = M grad, T, Y^n -> R2C] [y combine] [x update] [y^-1]
//              [z C2R -> clamp/store, zero-mode moments]
// Mathematically identical to the reference sequence (every dealias mask,
// the Laplacian and the Y^n transform folded into the linear spectral
// filters; see the op comments), with Y carried as Y_f + c where the scalar
// offset c (FP64) absorbs the zero-mode shift.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "dfloat.cuh"
#include "fft.cuh"
#include "fft246.cuh"
#include "dft41_tc.cuh"
#include "physics.cuh"

const char *pfgb_error_buffer(void);

// ---------------------------------------------------------------------------
// device state
// ---------------------------------------------------------------------------
struct KTab {
    const double *kx, *ky, *kz;
    const unsigned char *mx, *my, *mz;   // 1 = removed by the 2/3 rule
    __device__ __forceinline__ bool cut(int i, int j, int k) const { return (mx[i] | my[j] | mz[k]) != 0; }
    __device__ __forceinline__ double k2(int i, int j, int k) const {
        double a = kx[i], b = ky[j], c = kz[k];
        return a * a + b * b + c * c;
    }
};

template <typename T, typename TE>
struct DevState {
    Grid3 g;
    KTab kt;
    T *phi_old, *phi_new, *eta_old, *eta_new, *Y, *dYdt;
    T *Yprev;           // Y_f at the start of the step (the elastic solve's Y)
    T *q, *qb, *divr;   // q split: matrix storage (1 - h) x, its value before transport, div J
    TE *sig[6];         // stored stress of the elastic solve (minimize only, else null)
    T *mge, *mlap;      // minimize: explicit phi drive and Lap(phi)
    TE *eps[6];
    cplx_t<T> *S[4];
    cplx_t<TE> *E[6], *U[3];
    double *partials;
    double *dscal;
    double Yc, dYoff;   // Y = Y_f + Yc ; dY/dt = dYdt_f + dYoff
};

// device scalar slots
enum { DS_MEAN_DY = 0, DS_RES_DIFF = 1, DS_RES_REF = 2, DS_ZM = 4, DS_BR = 12, DS_EV = 16, DS_N = 24 };
// elastic-iteration status on the device (slots of the same array): done,
// updates taken, non-finite residual, converged.  While `done` is set, the
// kernels of further iterations launched ahead return at once.
enum { DS_EL = 56 };

struct pfgb_ctx {
    pfgb_params p;
    int device = 0;
    cudaStream_t stream = 0;
    // read-back: a side stream and two events (created on first use) let the
    // FP64 composition export run beside the copies of the other fields
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_rd[2] = {nullptr, nullptr};
    Grid3 g;
    AxisPlan plx, ply, plz;
    void *tw[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};  // [fp64|fp32][x,y,z]
    double *kx = nullptr, *ky = nullptr, *kz = nullptr;
    unsigned char *mx = nullptr, *my = nullptr, *mz = nullptr;
    void *phi[2] = {nullptr, nullptr}, *eta[2] = {nullptr, nullptr}, *Y = nullptr, *dYdt = nullptr;
    void *Yprev = nullptr;   // Y_f of the last step's start, for the stress export
    void *q = nullptr, *qb = nullptr, *divr = nullptr;   // q split state (pf_y_update_mode q)
    int q_rejected = 0, q_redistributed = 0;             // of the last step
    int gp_limited = 0;                                  // GP eta limiter: cells limited in the last step
    double *cstore = nullptr, *cmu = nullptr;            // conservative modes: storage and mu (FP64)
    int cons_limited = 0, cons_constrained = 0;          // of the last step
    int cur = 0, ecur = 0;
    void *S[4] = {nullptr, nullptr, nullptr, nullptr};
    void *eps[6] = {}, *E[6] = {}, *U[3] = {};
    double *partials = nullptr, *dscal = nullptr, *hscal = nullptr;
    double *stage = nullptr;          // host<->device staging, 5 N doubles, lazily allocated
    size_t npartials = 0;
    double Yc = 0.0, dYoff = 0.0, target_mass = 0.0;
    double Yc_prev = 0.0;    // Yc at the last step's start
    bool f246[3] = {false, false, false};   // x, y, z elastic passes on the 246-point engine
    // minimize state (mode = minimize)
    void *sig[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    void *Rk[3] = {nullptr, nullptr, nullptr}, *Dk[3] = {nullptr, nullptr, nullptr};   // increment form
    // Chebyshev semi-iteration of the increment: the previous iterate, the
    // relaxation gam = 2 / (2 - a - b) and sig = (b - a) / (2 - a - b) from
    // the spectral bounds [a, b] of the linear part; rho of the next update
    void *Dkm[3] = {nullptr, nullptr, nullptr};
    double cheb_gam = 1.0, cheb_sig = 0.0, cheb_rho = 1.0;
    // extrapolated warm start: u of the 1 to 5 steps before (as many levels
    // as the extrapolation order)
    void *Uhist[5][3] = {};
    int warm_count = 0;
    // learned start (elastic_warm_start_source 1, 2) and training pairs
    pfgb_fno *fno = nullptr;
    float *fno_in = nullptr, *fno_out = nullptr;     // [8][N], [3][N]
    void *Uhom[3] = {nullptr, nullptr, nullptr};     // u_hom of a training pair's cold start
    int pair_mode = 0;
    void *mge = nullptr, *mlap = nullptr;
    double lambda_vol = 0.0, V0_target = 0.0, prev_F_total = NAN;
    int min_iter = 0, conv_count = 0, converged_iter = 0, xb_clamp = 0;
    double sum_alpha = 0.0;   // sum (1 - h) of the last phi (zero-mode curvature bound)
    int warm_valid = 0, step = 0, loaded = 0;
    // runtime state a checkpoint carries: the last zero-mode solve and the
    // last elastic solve
    double zm_lambda = 0.0, zm_residual = 0.0, zm_derivative = 0.0;
    uint64_t zm_iterations = 0, zm_accepted = 0;
    uint64_t el_iterations = 0;
    double el_residual = 0.0;
    size_t bytes = 0;
    std::string err;
    PhysC pc;
    // launch accounting / optional per-kernel event timing
    long long launches = 0;
    int prof = 0;
    struct Rec { const char *tag; cudaEvent_t a, b; double bytes; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    size_t pool_used = 0;
    // while an elastic solve runs: &dscal[DS_EL] (its kernels return at once
    // once the device has decided the solve), else null
    const double *skip = nullptr;
    int last_el_iters = 0;   // updates of the last solve: the first batch launched ahead
    // tensor-core 41-point stage (fft_tensor_cores): its B table (hi | lo in
    // the shared-memory layout of dft41_tc.cuh) and a device error word set
    // when a bounded wait on the tensor core runs out
    void *tc_btab = nullptr;
    int *tc_err = nullptr;
    bool tc_y = false, tc_x = false, tc_z = false;   // passes that use it
};

// tag + algorithmic bytes of the next launch (set by the op-level wrappers)
struct LaunchTag { const char *tag; double bytes; };

static cudaEvent_t prof_event(pfgb_ctx *c) {
    if (c->pool_used == c->pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        c->pool.push_back(e);
    }
    return c->pool[c->pool_used++];
}

struct ProfScope {
    pfgb_ctx *c; LaunchTag t; cudaEvent_t a = nullptr;
    ProfScope(pfgb_ctx *c_, LaunchTag t_) : c(c_), t(t_) {
        c->launches++;
        if (c->prof && (a = prof_event(c))) cudaEventRecord(a, c->stream);
    }
    ~ProfScope() {
        if (c->prof && a) {
            cudaEvent_t b = prof_event(c);
            if (b) {
                cudaEventRecord(b, c->stream);
                c->recs.push_back({t.tag, a, b, t.bytes});
            }
        }
    }
};

// ---------------------------------------------------------------------------
// launch helpers
// ---------------------------------------------------------------------------
static const size_t kSmemBudget = 112 * 1024;
// strided-axis tiles narrower than 4 columns (8 bytes each) leave half of
// every 32-byte DRAM sector unused; long axes take 4 columns at one block
// per SM instead, up to this budget
static const size_t kSmemWide = 220 * 1024;

// The dynamic shared-memory limit is an attribute of the kernel function,
// shared by every context in the process: it is raised to the device's
// opt-in maximum (the same value from every thread), never set to one
// launch's size, so contexts of different grids can launch concurrently.
static int smem_optin_max() {
    static std::atomic<int> v(0);
    int m = v.load();
    if (m == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&m, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || m <= 0)
            m = 227 * 1024;
        v.store(m);
    }
    return m;
}
static std::mutex g_smem_mu;
static std::map<std::pair<int, const void *>, int> g_smem_limit;   // (device, kernel) -> dynamic limit

template <typename K>
static cudaError_t allow_smem(K kernel, size_t bytes) {
    if (bytes <= 48 * 1024) return cudaSuccess;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_pair(dev, (const void *)kernel);
    std::lock_guard<std::mutex> lk(g_smem_mu);
    auto it = g_smem_limit.find(key);
    if (it == g_smem_limit.end()) {
        // static + dynamic shared memory may not exceed the opt-in maximum
        cudaFuncAttributes fa;
        if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
        const int m = smem_optin_max() - (int)fa.sharedSizeBytes;
        if ((e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, m)) != cudaSuccess) return e;
        it = g_smem_limit.emplace(key, m).first;
    }
    return (int)bytes <= it->second ? cudaSuccess : cudaErrorInvalidValue;
}

template <typename T>
static const cplx_t<T> *twp(const pfgb_ctx *c, int axis) {
    return (const cplx_t<T> *)c->tw[sizeof(T) == 8 ? 0 : 1][axis];
}

// ---------------------------------------------------------------------------
// tile autotuner of the generic engine (fft_autotune = 1): the columns per
// block of an x or y pass (TK, a power of two) and the rows per block of a z
// pass (R) are timed over their candidates on first use, and the fastest is
// kept per kernel, grid shape and device for the life of the process (a
// sweep of many cases tunes each grid size once).  An axis pass is timed as
// itself on scratch arrays (its ops are pure functions of their inputs); a
// z pass, whose ops write the step's fields, through a copy op with the
// same field counts.  Two threads may tune the same key at once; the first
// result stored stands.  pfgb_batch_minimize tunes each distinct grid on
// one thread before its workers start, on an otherwise idle device.
// ---------------------------------------------------------------------------
struct TileKey {
    int dev;
    const void *kern;
    long long a, b, c;
    bool operator<(const TileKey &o) const {
        if (dev != o.dev) return dev < o.dev;
        if (kern != o.kern) return kern < o.kern;
        if (a != o.a) return a < o.a;
        if (b != o.b) return b < o.b;
        return c < o.c;
    }
};
struct TileRec { int tile, rule; float t_ms, t_rule_ms; std::string tag; long long a, b, c; };
static std::mutex g_tile_mu;
static std::map<TileKey, TileRec> g_tiles;

// zeroed scratch arrays of `bytes` each, stream-ordered (no device-wide
// synchronisation while other contexts run), freed with the object
struct TuneScratch {
    std::vector<void *> p;
    cudaStream_t s;
    bool ok = true;
    TuneScratch(const TuneScratch &) = delete;
    TuneScratch &operator=(const TuneScratch &) = delete;
    TuneScratch(int n, size_t bytes, cudaStream_t st) : s(st) {
        for (int i = 0; i < n && ok; ++i) {
            void *q = nullptr;
            ok = cudaMallocAsync(&q, bytes, s) == cudaSuccess;
            if (ok) ok = cudaMemsetAsync(q, 0, bytes, s) == cudaSuccess;
            p.push_back(q);
        }
    }
    ~TuneScratch() {
        for (void *q : p)
            if (q) cudaFreeAsync(q, s);
    }
};

// the number of copies of a candidate timed together: the concurrency of
// the caller's cases (pfgb_batch_minimize sets it while it tunes), so the
// choice is the one with the best throughput on a device the cases share
static std::atomic<int> g_tune_copies(1);

// one warm-up round, then the best of three (ms per round); a round is one
// launch on each of the given streams, forked from and joined to the
// first; infinity if a launch fails
template <typename F>
static float time_launch(const std::vector<cudaStream_t> &ss, F &&launch) {
    const int k = (int)ss.size();
    std::vector<cudaEvent_t> ev(k + 1, nullptr);
    float best = INFINITY;
    bool ok = true;
    for (auto &e : ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDefault) == cudaSuccess;
    auto round = [&](bool timed) {
        if (timed) cudaEventRecord(ev[0], ss[0]);
        else cudaEventRecord(ev[k], ss[0]);
        for (int i = 1; i < k; ++i) cudaStreamWaitEvent(ss[i], timed ? ev[0] : ev[k], 0);
        for (int i = 0; i < k; ++i) launch(i);
        for (int i = 1; i < k; ++i) {
            cudaEventRecord(ev[i], ss[i]);
            cudaStreamWaitEvent(ss[0], ev[i], 0);
        }
        cudaEventRecord(ev[k], ss[0]);
    };
    if (ok) {
        round(false);
        if (cudaGetLastError() == cudaSuccess) {
            for (int r = 0; r < 3; ++r) {
                round(true);
                if (cudaEventSynchronize(ev[k]) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
                    best = INFINITY;
                    break;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ev[0], ev[k]);
                best = std::min(best, ms);
            }
        }
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    return best;
}

// the context's stream and g_tune_copies - 1 more, each with its own
// scratch arrays
struct TuneStreams {
    std::vector<cudaStream_t> ss;
    std::vector<std::unique_ptr<TuneScratch>> sc;
    bool ok = true;
    TuneStreams(cudaStream_t s0, int narr, size_t bytes) {
        const int k = std::max(1, std::min(16, g_tune_copies.load()));
        for (int i = 0; i < k && ok; ++i) {
            cudaStream_t s = s0;
            if (i > 0) ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
            if (!ok) break;
            ss.push_back(s);
            sc.push_back(std::make_unique<TuneScratch>(narr, bytes, s));
            ok = sc.back()->ok;
        }
    }
    TuneStreams(const TuneStreams &) = delete;
    TuneStreams &operator=(const TuneStreams &) = delete;
    ~TuneStreams() {
        sc.clear();   // stream-ordered frees first
        if (!ss.empty()) cudaStreamSynchronize(ss[0]);
        for (size_t i = 1; i < ss.size(); ++i) {
            cudaStreamSynchronize(ss[i]);
            cudaStreamDestroy(ss[i]);
        }
    }
};



// copy op of a z pass with NFI fields in and NFO out, for timing its tiles
template <typename T, int NFI, int NFO>
struct OpTuneZ {
    using Acc = NoAcc;
    const cplx_t<T> *src[NFI > 0 ? NFI : 1];
    cplx_t<T> *dst[NFO > 0 ? NFO : 1];
    int NzC;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const {
#pragma unroll
        for (int f = 0; f < NFI; ++f) v[f] = src[f][row * NzC + k];
    }
    __device__ void point(long long, const T *in, T *out, Acc &) const {
#pragma unroll
        for (int f = 0; f < NFO; ++f) out[f] = NFI > 0 ? in[f % (NFI > 0 ? NFI : 1)] : T(0);
    }
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
#pragma unroll
        for (int f = 0; f < NFO; ++f) dst[f][row * NzC + k] = v[f];
    }
};

template <typename T, int NIN, int NOUT, int DIN, int DOUT, class Op>
static int tuned_tk(pfgb_ctx *c, int axis, const AxisPlan &pl, const Op &op, int rule, const char *tag) {
    using T2 = cplx_t<T>;
    auto kern = k_axis_pass<T, NIN, NOUT, DIN, DOUT, Op>;
    int dev = 0;
    cudaGetDevice(&dev);
    const int gy = axis == 1 ? c->g.Nx : c->g.Ny;
    const TileKey key{dev, (const void *)kern, pl.n, c->g.NzC, gy};
    {
        std::lock_guard<std::mutex> lk(g_tile_mu);
        auto it = g_tiles.find(key);
        if (it != g_tiles.end()) return it->second.tile;
    }
    constexpr int NW = axis_width<NIN, NOUT>();
    const int n = pl.n;
    auto bytes = [&](int tk) { return ((size_t)n + 2 * (size_t)n * (NW * tk + 1)) * sizeof(T2); };
    TileRec rec{rule, rule, INFINITY, INFINITY, tag, n, c->g.NzC, gy};
    {
        TuneStreams ts(c->stream, NIN + NOUT, (size_t)c->g.Nk * sizeof(T2));
        if (ts.ok) {
            std::vector<AxisIO<T, NIN, NOUT>> io(ts.ss.size());
            for (size_t i = 0; i < io.size(); ++i) {
                for (int a = 0; a < NIN; ++a) io[i].in[a] = (const T2 *)ts.sc[i]->p[a];
                for (int b = 0; b < NOUT; ++b) io[i].out[b] = (T2 *)ts.sc[i]->p[NIN + b];
            }
            for (int tk = 1; tk <= 32; tk <<= 1) {
                if (tk > 1 && tk / 2 >= c->g.NzC) break;
                const size_t smem = bytes(tk);
                if (smem > kSmemWide || allow_smem(kern, smem) != cudaSuccess) break;
                const dim3 grid((c->g.NzC + tk - 1) / tk, gy);
                const T2 *tw = twp<T>(c, axis == 1 ? 1 : 0);
                const float t = time_launch(ts.ss, [&](int i) {
                    kern<<<grid, 256, smem, ts.ss[i]>>>(c->g, axis, pl, tw, tk, io[i], op, nullptr);
                });
                if (tk == rule) rec.t_rule_ms = t;
                if (t < rec.t_ms) { rec.t_ms = t; rec.tile = tk; }
            }
        }
    }
    cudaGetLastError();   // a candidate that could not launch is not chosen
    std::lock_guard<std::mutex> lk(g_tile_mu);
    return g_tiles.emplace(key, rec).first->second.tile;   // the first thread's choice stands
}

// shared memory of a generic z pass of R rows of length n
template <typename T, int NFI, int NFO>
static size_t zpass_bytes(int R, int n) {
    int PI_ = NFI > 0 ? (R * NFI + 1) / 2 : 0, PO_ = NFO > 0 ? (R * NFO + 1) / 2 : 0;
    if (NFI == NFO) PO_ = 0;   // in-place pointwise stage
    return ((size_t)n + 2 * (size_t)PI_ * n + 2 * (size_t)PO_ * n) * sizeof(cplx_t<T>);
}

template <typename T, int NFI, int NFO>
static int tuned_r(pfgb_ctx *c, int rule, size_t (*bytes)(int, int), const char *tag) {
    using T2 = cplx_t<T>;
    using OpT = OpTuneZ<T, NFI, NFO>;
    auto kern = k_zpass<T, NFI, NFO, OpT>;
    int dev = 0;
    cudaGetDevice(&dev);
    const long long rows = (long long)c->g.Nx * c->g.Ny;
    const TileKey key{dev, (const void *)kern, c->g.Nz, rows, 0};
    {
        std::lock_guard<std::mutex> lk(g_tile_mu);
        auto it = g_tiles.find(key);
        if (it != g_tiles.end()) return it->second.tile;
    }
    TileRec rec{rule, rule, INFINITY, INFINITY, tag, c->g.Nz, rows, 0};
    {
        TuneStreams ts(c->stream, NFI + NFO, (size_t)c->g.Nk * sizeof(T2));
        if (ts.ok) {
            std::vector<OpT> op(ts.ss.size());
            for (size_t i = 0; i < op.size(); ++i) {
                for (int f = 0; f < NFI; ++f) op[i].src[f] = (const T2 *)ts.sc[i]->p[f];
                for (int f = 0; f < NFO; ++f) op[i].dst[f] = (T2 *)ts.sc[i]->p[NFI + f];
                op[i].NzC = c->g.NzC;
            }
            for (int r = 2; r <= 128; r <<= 1) {
                if (r / 2 >= rows) break;
                const size_t smem = bytes(r, c->g.Nz);
                if (smem > kSmemWide || allow_smem(kern, smem) != cudaSuccess) break;
                const int nb = (int)((rows + r - 1) / r);
                const T2 *tw = twp<T>(c, 2);
                const float t = time_launch(ts.ss, [&](int i) {
                    kern<<<nb, 256, smem, ts.ss[i]>>>(c->g, c->plz, tw, r, op[i], nullptr);
                });
                if (r == rule) rec.t_rule_ms = t;
                if (t < rec.t_ms) { rec.t_ms = t; rec.tile = r; }
            }
        }
    }
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(g_tile_mu);
    return g_tiles.emplace(key, rec).first->second.tile;
}

template <typename T, int NIN, int NOUT, int DIN, int DOUT, class Op>
static pfgb_status launch_axis(pfgb_ctx *c, int axis, AxisIO<T, NIN, NOUT> io, Op op, const char *tag) {
    using T2 = cplx_t<T>;
    const AxisPlan &pl = axis == 1 ? c->ply : c->plx;
    const int n = pl.n;
    if constexpr (std::is_same<T, float>::value && f246_axis_fits<NIN, NOUT>()) {
        // 246-long FP32 axes with an even half-spectrum row: the 6 x 41 engine
        if (n == f246::N && c->g.NzC % 2 == 0) {
            constexpr int TCW = f246::NL / axis_width<NIN, NOUT>();
            const size_t smem = f246::axis_smem_bytes();
            auto kern = k_axis246<NIN, NOUT, DIN, DOUT, Op>;
            PFGB_CUDA_TRY(allow_smem(kern, smem));
            dim3 grid((c->g.NzC + TCW - 1) / TCW, axis == 1 ? c->g.Nx : c->g.Ny);
            ProfScope ps(c, {tag, (double)(NIN + NOUT) * (double)c->g.Nk * sizeof(T2)});
            kern<<<grid, f246::THREADS, smem, c->stream>>>(c->g, axis, (const float2 *)twp<T>(c, axis == 1 ? 1 : 0),
                                                         io, op, c->skip);
            PFGB_CUDA_TRY(cudaGetLastError());
            return PFGB_OK;
        }
    }
    constexpr int NW = axis_width<NIN, NOUT>();
    auto bytes = [&](int tk) { return ((size_t)n + 2 * (size_t)n * (NW * tk + 1)) * sizeof(T2); };
    int TK = 16;
    while (TK > 1 && bytes(TK) > kSmemBudget) TK >>= 1;
    if (TK < 4 && sizeof(T) == 4 && bytes(4) <= kSmemWide) TK = 4;
    while (TK > 1 && TK / 2 >= c->g.NzC) TK >>= 1;
    if (c->p.fft_autotune & 1) TK = tuned_tk<T, NIN, NOUT, DIN, DOUT, Op>(c, axis, pl, op, TK, tag);
    const size_t smem = bytes(TK);
    auto kern = k_axis_pass<T, NIN, NOUT, DIN, DOUT, Op>;
    PFGB_CUDA_TRY(allow_smem(kern, smem));
    dim3 grid((c->g.NzC + TK - 1) / TK, axis == 1 ? c->g.Nx : c->g.Ny);
    ProfScope ps(c, {tag, (double)(NIN + NOUT) * (double)c->g.Nk * sizeof(T2)});
    kern<<<grid, 256, smem, c->stream>>>(c->g, axis, pl, twp<T>(c, axis == 1 ? 1 : 0), TK, io, op, c->skip);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// generic z pass on the 246-point engine: NFI half spectra per row in
// (Hermitian-packed two per complex line), C2R, the op's pointwise stage,
// R2C, NFO half spectra out.  A row takes LW = max(ceil(NFI/2), ceil(NFO/2))
// lines, a block NL / LW rows.
template <int NFI, int NFO>
constexpr bool f246_z_fits() {
    constexpr int LI = (NFI + 1) / 2, LO = (NFO + 1) / 2, LW = LI > LO ? LI : LO;
    return LW >= 1 && LW <= 3;
}

template <int NFI, int NFO, class Op>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_zpass246g(Grid3 g, const float2 *tw_g, Op op, const double *skip) {
    if (skip && *skip != 0.0) return;
    using namespace f246;
    constexpr int LI = (NFI + 1) / 2, LO = (NFO + 1) / 2, LW = LI > LO ? LI : LO;
    constexpr int R = NL / LW, NC = N / 2 + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *buf = tw + N;
    const long long row0 = (long long)blockIdx.x * R;
    const long long nrows = (long long)g.Nx * g.Ny;
    const int rcnt = (int)min((long long)R, nrows - row0);
    load_twiddles(tw, tw_g);
    if constexpr (NFI > 0) {
#pragma unroll 2
        for (int e = threadIdx.x; e < R * NC; e += blockDim.x) {
            const int rr = e / NC, k = e - rr * NC;
            float2 v[NFI];
            if (rr < rcnt) op.load_spec(row0 + rr, k, v);
            else {
#pragma unroll
                for (int f = 0; f < NFI; ++f) v[f] = make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int f = 0; f < LI; ++f) {
                float2 Av = v[2 * f], Bv = 2 * f + 1 < NFI ? v[2 * f + 1] : make_float2(0.f, 0.f);
                if (k == 0 || 2 * k == N) { Av.y = 0.f; Bv.y = 0.f; }
                float2 *line = buf + (rr * LW + f) * N;
                // Z_k = A_k + i B_k ; Z_(n-k) = conj(A_k) + i conj(B_k)
                line[k] = make_float2(Av.x - Bv.y, Av.y + Bv.x);
                if (k > 0 && 2 * k != N) line[N - k] = make_float2(Av.x + Bv.y, Bv.x - Av.y);
            }
        }
        __syncthreads();
        lines<+1, 1, N>(buf, tw);
    } else {
        __syncthreads();   // twiddles
    }
    typename Op::Acc acc = Op::Acc::identity();
    auto cell_step = [&](int e, auto &&pointf) {
        const int r = e / N, z = e - r * N;
        float vi[NFI > 0 ? NFI : 1], vo[NFO > 0 ? NFO : 1];
#pragma unroll
        for (int f = 0; f < NFI; ++f) {
            const float2 w = buf[(r * LW + f / 2) * N + z];
            vi[f] = (f & 1) ? w.y : w.x;
        }
        pointf((row0 + r) * N + z, vi, vo);
#pragma unroll
        for (int f = 0; f < LO; ++f)
            buf[(r * LW + f) * N + z] = make_float2(vo[2 * f], 2 * f + 1 < NFO ? vo[2 * f + 1] : 0.f);
    };
    constexpr int B = op_batch<Op>::value;
    if constexpr (B > 1) {
        for (int e0 = threadIdx.x; e0 < rcnt * N; e0 += B * blockDim.x) {
            typename Op::Pre pre[B];
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int e = e0 + b * blockDim.x;
                if (e < rcnt * N) op.fetch(row0 * N + e, pre[b]);
            }
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int e = e0 + b * blockDim.x;
                if (e < rcnt * N)
                    cell_step(e, [&](long long cell, const float *vi, float *vo) { op.point_with(cell, pre[b], vi, vo, acc); });
            }
        }
    } else {
        for (int e = threadIdx.x; e < rcnt * N; e += blockDim.x)
            cell_step(e, [&](long long cell, const float *vi, float *vo) { op.point(cell, vi, vo, acc); });
    }
    if constexpr (Op::Acc::kActive) {
        block_reduce_acc(acc);
        if (threadIdx.x == 0) op.finish(blockIdx.x, acc);
    }
    if constexpr (NFO > 0) {
        __syncthreads();
        lines<-1, 1, N>(buf, tw);
        for (int e = threadIdx.x; e < rcnt * NC; e += blockDim.x) {
            const int rr = e / NC, k = e - rr * NC;
            float2 v[NFO];
#pragma unroll
            for (int f = 0; f < LO; ++f) {
                const float2 *line = buf + (rr * LW + f) * N;
                const float2 Zk = line[k], Zm = line[k == 0 ? 0 : N - k];
                // A_k = (Z_k + conj Z_-k) / 2 ; B_k = (Z_k - conj Z_-k) / (2 i)
                v[2 * f] = make_float2(0.5f * (Zk.x + Zm.x), 0.5f * (Zk.y - Zm.y));
                if (2 * f + 1 < NFO) v[2 * f + 1] = make_float2(0.5f * (Zk.y + Zm.y), 0.5f * (Zm.x - Zk.x));
            }
            op.store_spec(row0 + rr, k, v);
        }
    }
}

// extra_bytes: field bytes the op reads/writes per call besides its NFI/NFO spectra
template <typename T, int NFI, int NFO, class Op>
static pfgb_status launch_z(pfgb_ctx *c, Op op, const char *tag, double extra_bytes, int *nblocks = nullptr) {
    using T2 = cplx_t<T>;
    const int n = c->g.Nz;
    if constexpr (std::is_same<T, float>::value && f246_z_fits<NFI, NFO>()) {
        if (n == f246::N) {   // 246-long FP32 rows: the 6 x 41 engine
            constexpr int LW = ((NFI + 1) / 2 > (NFO + 1) / 2) ? (NFI + 1) / 2 : (NFO + 1) / 2;
            constexpr int R = f246::NL / LW;
            const size_t smem = f246::z_smem_bytes();
            auto kern = k_zpass246g<NFI, NFO, Op>;
            PFGB_CUDA_TRY(allow_smem(kern, smem));
            const long long rows = (long long)c->g.Nx * c->g.Ny;
            const int nb = (int)((rows + R - 1) / R);
            ProfScope ps(c, {tag, (double)(NFI + NFO) * (double)c->g.Nk * sizeof(T2) + extra_bytes});
            kern<<<nb, f246::THREADS, smem, c->stream>>>(c->g, (const float2 *)twp<T>(c, 2), op, c->skip);
            PFGB_CUDA_TRY(cudaGetLastError());
            if (nblocks) *nblocks = nb;
            return PFGB_OK;
        }
    }
    auto bytes = [&](int R) { return zpass_bytes<T, NFI, NFO>(R, n); };
    int R = 64;
    while (R > 2 && bytes(R) > kSmemBudget) R >>= 1;
    const long long rows = (long long)c->g.Nx * c->g.Ny;
    while (R > 2 && R / 2 >= rows) R >>= 1;
    if (c->p.fft_autotune & 2) R = tuned_r<T, NFI, NFO>(c, R, &zpass_bytes<T, NFI, NFO>, tag);
    const size_t smem = bytes(R);
    auto kern = k_zpass<T, NFI, NFO, Op>;
    PFGB_CUDA_TRY(allow_smem(kern, smem));
    const int nb = (int)((rows + R - 1) / R);
    ProfScope ps(c, {tag, (double)(NFI + NFO) * (double)c->g.Nk * sizeof(T2) + extra_bytes});
    kern<<<nb, 256, smem, c->stream>>>(c->g, c->plz, twp<T>(c, 2), R, op, c->skip);
    PFGB_CUDA_TRY(cudaGetLastError());
    if (nblocks) *nblocks = nb;
    return PFGB_OK;
}

#define TRY(x)                                   \
    do {                                         \
        pfgb_status s_ = (x);                    \
        if (s_ != PFGB_OK) return s_;            \
    } while (0)

// ---------------------------------------------------------------------------
// reductions of block partials (fixed order -> deterministic)
// ---------------------------------------------------------------------------
struct AccSum1 {
    static constexpr bool kActive = true;
    double s;
    __device__ static AccSum1 identity() { return {0.0}; }
    __device__ static AccSum1 combine(AccSum1 a, AccSum1 b) { return {a.s + b.s}; }
    __device__ static AccSum1 shfl_down(AccSum1 a, int o) { return {__shfl_down_sync(0xffffffffu, a.s, o)}; }
};
struct AccSum2 {
    static constexpr bool kActive = true;
    double a, b;
    __device__ static AccSum2 identity() { return {0.0, 0.0}; }
    __device__ static AccSum2 combine(AccSum2 x, AccSum2 y) { return {x.a + y.a, x.b + y.b}; }
    __device__ static AccSum2 shfl_down(AccSum2 x, int o) {
        return {__shfl_down_sync(0xffffffffu, x.a, o), __shfl_down_sync(0xffffffffu, x.b, o)};
    }
};
// zero-mode statistics: min, max of Y*, and the Taylor moments
// M_p = sum (1-h) sigma^{(p)}(Y*) (M_0 also + h v_B), p = 0..4
// (m[5] = sum |1 - h|, the curvature bound of the zero-mode certification).
// Per-thread and per-block sums in FP32 (AccZMf, predictor / bound only),
// block partials widened to FP64 for the grid reduction (AccZM).
template <typename R>
struct AccZMt {
    static constexpr bool kActive = true;
    R mn, mx, m[6];
    __device__ static AccZMt identity() { return {R(3e38), R(-3e38), {0, 0, 0, 0, 0, 0}}; }
    __device__ static AccZMt combine(AccZMt x, const AccZMt &y) {
        x.mn = fmin(x.mn, y.mn);
        x.mx = fmax(x.mx, y.mx);
#pragma unroll
        for (int i = 0; i < 6; ++i) x.m[i] += y.m[i];
        return x;
    }
    __device__ static AccZMt shfl_down(AccZMt x, int o) {
        AccZMt r;
        r.mn = __shfl_down_sync(0xffffffffu, x.mn, o);
        r.mx = __shfl_down_sync(0xffffffffu, x.mx, o);
#pragma unroll
        for (int i = 0; i < 6; ++i) r.m[i] = __shfl_down_sync(0xffffffffu, x.m[i], o);
        return r;
    }
};
using AccZM = AccZMt<double>;

template <class Acc>
__global__ void k_reduce_partials(const Acc *part, int n, double *out, int slot, double scale,
                                  const double *skip = nullptr) {
    if (skip && *skip != 0.0) return;
    Acc a = Acc::identity();
    for (int i = threadIdx.x; i < n; i += blockDim.x) a = Acc::combine(a, part[i]);
    block_reduce_acc(a);
    if (threadIdx.x == 0) {
        const double *v = reinterpret_cast<const double *>(&a);
        for (int i = 0; i < (int)(sizeof(Acc) / sizeof(double)); ++i) out[slot + i] = v[i] * scale;
    }
}

template <class Acc>
static pfgb_status reduce_to(pfgb_ctx *c, int nblocks, int slot, double scale = 1.0) {
    ProfScope ps(c, {"reduce_partials", (double)nblocks * sizeof(Acc)});
    k_reduce_partials<Acc><<<1, 256, 0, c->stream>>>((const Acc *)c->partials, nblocks, c->dscal, slot, scale,
                                                     c->skip);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// ===========================================================================
// phi / eta Allen-Cahn updates
//   reference: D2Z f -> dealias; rhs -> D2Z -> dealias;
//   f_k <- (f_k - L dt rhs_k) / (1 + L dt kappa k^2); dealias; Z2D; /N; clamp
//   here: transform (f - L dt rhs) once (linearity), one mask, /N folded in.
// ===========================================================================
template <typename T, typename TE>
struct OpPhiR2C {   // z pass producer: phi - L dt rhs_phi
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec;
    // the fields of two cells read ahead of their work
    static constexpr int kBatch = 2;
    struct Pre { T phi, Y, eta; TE e[6]; };
    __device__ void fetch(long long cell, Pre &p) const {
        p.phi = d.phi_old[cell];
        p.Y = d.Y[cell];
        p.eta = c.gp ? d.eta_old[cell] : T(0);
        if (c.coupling) {
#pragma unroll
            for (int a = 0; a < 6; ++a) p.e[a] = d.eps[a][cell];
        }
    }
    __device__ void point(long long cell, const T *in, T *out, Acc &acc) const {
        Pre p;
        fetch(cell, p);
        point_with(cell, p, in, out, acc);
    }
    __device__ void point_with(long long, const Pre &p, const T *, T *out, Acc &) const {
        const T xB = xB_of_Y<T>(c, p.Y + T(d.Yc));
        const T r = phi_rhs<T, TE>(c, ec, p.phi, p.eta, xB, p.e);
        out[0] = p.phi - T(c.Ldt) * r;
    }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        d.S[0][row * d.g.NzC + k] = v[0];
    }
};

template <typename T, typename TE>
struct OpEtaR2C {   // z pass producer: eta - L_eta dt rhs_eta (phi = updated phi)
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec;
    __device__ void point(long long cell, const T *, T *out, Acc &) const {
        const T eta = d.eta_old[cell];
        const T phi = d.phi_new[cell];
        const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
        T sh = 0;
        if (c.gp_el && c.act_eta && c.elastic) {
            TE e[6], s[6];
#pragma unroll
            for (int a = 0; a < 6; ++a) e[a] = d.eps[a][cell];
            stress_at<T, TE>(c, ec, d.phi_old[cell], eta, xB, e, s);
            sh = T(s[0]) + T(s[1]) + T(s[2]);
        }
        const T r = eta_rhs<T, TE>(c, ec, eta, phi, xB, sh);
        out[0] = eta - T(c.gpLdt) * r;
    }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        d.S[0][row * d.g.NzC + k] = v[0];
    }
};

template <typename T>
struct OpACFilterX {   // x pass: mask / (1 + L dt kappa k^2) / N
    static constexpr bool kInplace = false;
    KTab kt; double Ldtk, invN;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        if (kt.cut(i, j, k)) { out[0] = mk2<cplx_t<T>>(T(0), T(0)); return; }
        const T f = T(invN / (1.0 + Ldtk * kt.k2(i, j, k)));
        out[0] = cscale(in[0], f);
    }
};

template <typename T, typename TE>
struct OpACStoreZ {   // z pass consumer: clamp and store the new order parameter
    using Acc = NoAcc;
    const cplx_t<T> *src; T *dst; int NzC; T lo, hi;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &) const {
        T v = in[0];
        if (v < lo) v = lo;
        if (v > hi) v = hi;
        dst[cell] = v;
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
};

// ===========================================================================
// Y (logit composition) update
// ===========================================================================
// (1) chemical potential mu (compute_mu_x_kernel :1266-1324 / compute_mu_C_gp
// :1326-1366) and sum of D_mix(h) xB (1-xB) (reduce_sum_DY_kernel :3870).
// GPC: the GP storage coupling's <DY> (a separate instance, so the other
// paths carry none of its code)
template <typename T, typename TE, bool GPC = false>
struct OpMuR2C {
    using Acc = AccSum1;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec;
    // the fields of two cells read ahead of their work
    static constexpr int kBatch = 2;
    struct Pre { T Y, po, pn, eta; TE e[6]; };
    __device__ void fetch(long long cell, Pre &p) const {
        p.Y = d.Y[cell];
        p.po = d.phi_old[cell];
        p.pn = (c.zm || c.prev_level) ? p.po : d.phi_new[cell];
        p.eta = (c.elastic && c.gp) ? d.eta_old[cell] : T(0);
        if (c.elastic) {
#pragma unroll
            for (int a = 0; a < 6; ++a) p.e[a] = d.eps[a][cell];
        }
    }
    __device__ void point(long long cell, const T *in, T *out, Acc &acc) const {
        Pre p;
        fetch(cell, p);
        point_with(cell, p, in, out, acc);
    }
    __device__ void point_with(long long cell, const Pre &p, const T *, T *out, Acc &acc) const {
        const T Yv = p.Y + T(d.Yc);
        const T phiY = p.pn;
        const T xB = sigmoid_clip(Yv, T(c.Yclip), T(c.xBeps));
        T offA, offB;
        thermo_mu_off<T>(c.tc, xB, offA, offB);
        T mu;
        if (c.gp) {
            const T cref = T(1) / (T(c.Vm0) + T(c.dVm) * xB);
            mu = cref * (T(c.dG) + offB - offA);
        } else {
            const T h = pf_h(phiY);
            const T cb = c_xB_phi<T>(xB, T(c.Vm0), T(c.dVm), T(c.Vmc), h);
            const T muA = T(c.tc.GA_s) + offA, muB = T(c.tc.GB_s) + offB;
            const T mt = (T(1) - h) * (muA * (T(1) - xB) + muB * xB) + h * T(c.mu0);
            mu = cb * ((T(c.dG) + offB - offA) - cb * mt * T(c.dVm));
        }
        if (c.elastic) {
            // stress of the elastic solve of this step: phi, eta, xB at step start
            TE s[6];
            const T xB0 = xB_of_Y<T>(c, Yv);
            stress_at<T, TE>(c, ec, p.po, p.eta, xB0, p.e, s);
            mu += -T(c.eiv) * (T(s[0]) + T(s[1]) + T(s[2]));
        }
        out[0] = mu;
        if constexpr (GPC) {
            // reduce_sum_DY_gp_kernel (:3923-3955): h_alpha D_alpha x (1 - x)
            // at eta_for_Y_explicit (main_cuda.cu:30292)
            const T hp = pf_h(phiY), he = pf_h(c.prev_level ? d.eta_old[cell] : d.eta_new[cell]);
            const T xs = sigmoid_clip(Yv, T(20), T(1e-12));
            acc.s += double((T(1) - hp) * (T(1) - he) * T(c.Da) * (xs * (T(1) - xs)));
            return;
        }
        const T h = pf_h(phiY);
        const T Dm = (T(1) - h) * T(c.Da) + h * T(c.Dc);
        T x = sigmoid_raw(Yv);
        if (x < T(1e-12)) x = T(1e-12);
        if (x > T(1) - T(1e-12)) x = T(1) - T(1e-12);
        acc.s += double(Dm * x * (T(1) - x));
    }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        d.S[0][row * d.g.NzC + k] = v[0];
    }
    __device__ void finish(int b, const Acc &a) const { reinterpret_cast<Acc *>(d.partials)[b] = a; }
};

// (2) gradient: g_a = IFFT(mask i k_a mask mu_k)/N, three outputs
template <typename T>
struct OpGradX {
    static constexpr bool kInplace = false;
    KTab kt; double invN;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        using T2 = cplx_t<T>;
        if (kt.cut(i, j, k)) { out[0] = out[1] = out[2] = mk2<T2>(T(0), T(0)); return; }
        const T2 m = cscale(in[0], T(invN));
        out[0] = cmul_is(m, T(kt.kx[i]));
        out[1] = cmul_is(m, T(kt.ky[j]));
        out[2] = cmul_is(m, T(kt.kz[k]));
    }
};

// (3) fused C2R of the gradients -> fluxes J = M grad mu, the explicit
// source T = term_h + term_gamma of the Y right-hand side
// (compute_Y_rhs_kernel :2185-2266 / _sm_tangent_n_ :2268-2359) and Y^n,
// then R2C.  The spectral side combines i kz J_z - T into one array.
// GPC: the GP storage coupling's source and the limiter's second flux (a
// separate instance, so the other paths carry none of their code)
template <typename T, typename TE, bool GPC = false>
struct OpFluxZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const {
        const long long o = row * d.g.NzC + k;
        v[0] = d.S[0][o]; v[1] = d.S[1][o]; v[2] = d.S[2][o];
    }
    // the five fields of four cells read ahead of their work
    static constexpr int kBatch = 4;
    struct Pre { T Y, pn, pp, eta, dydt; };
    __device__ void fetch(long long cell, Pre &p) const {
        p.Y = d.Y[cell];
        p.pn = d.phi_old[cell];
        p.pp = d.phi_new[cell];
        p.eta = c.gp ? d.eta_new[cell] : T(0);
        p.dydt = d.dYdt[cell];
    }
    __device__ void point(long long cell, const T *g, T *out, Acc &acc) const {
        Pre p;
        fetch(cell, p);
        point_with(cell, p, g, out, acc);
    }
    __device__ void point_with(long long cell, const Pre &p, const T *g, T *out, Acc &) const {
        const T Yf = p.Y;
        const T Yv = Yf + T(d.Yc);
        const T pn = p.pn, pp = p.pp;
        const T phiY = (c.zm || c.prev_level) ? pn : pp;
        const T xBp = sigmoid_clip(Yv, T(c.Yclip), T(c.xBeps));
        // q split: the matrix channel alone, (1 - h) M_alpha with G_alpha at
        // h = 0 (compute_flux_single_component_q_kernel, cuda_kernels.cu:2014-2037)
        T M;
        if (GPC && xmob) {
            // the GP mobility at the composition held in xmob, in FP64 as the
            // reference evaluates it (compute_flux_single_component_gp_kernel,
            // cuda_kernels.cu:2039-2071; outside [0, 1] its difference quotient
            // is not finite and the mobility takes its cap)
            const double hb = pf_h(double(phiY)), he = pf_h(double(p.eta));
            const double Ga = gamma_thermo<double>(tcd, double(xmob[cell]), 0.0, md[0], md[1], md[2]);
            const double Ma = stabilized_meff<double>(md[3], Ga);
            M = T((1.0 - hb) * (1.0 - he) * Ma + (1.0 - hb) * he * md[4] + hb * md[5]);
        } else {
            M = qmob ? (T(1) - pf_h(clamp01(phiY))) *
                           stabilized_meff<T>(T(c.Da), gamma_thermo<T>(c.tc, xBp, T(0), T(c.Vm0), T(c.dVm),
                                                                        T(c.Vmc)))
                     : mobility<T>(c, phiY, p.eta, xBp);
        }
        out[0] = M * g[0];
        out[1] = M * g[1];
        out[2] = M * g[2];
        T x = sigmoid_raw(Yv);
        if (x < T(1e-12)) x = T(1e-12);
        if (x > T(1) - T(1e-12)) x = T(1) - T(1e-12);
        const T ld = x * (T(1) - x);
        const T dYdt = p.dydt + T(d.dYoff);
        const T dt = T(c.dt);
        T src;
        if (GPC) {
            // GP storage source and gamma term (compute_Y_rhs_gp_kernel
            // :2361-2430; conservative_y_rhs :2432-2527 without the floor)
            const T hpn = pf_h(pp), hen = pf_h(p.eta), hpo = pf_h(pn), heo = pf_h(d.eta_old[cell]);
            const T hgn = (T(1) - hpn) * hen, hgo = (T(1) - hpo) * heo;
            const T han = (T(1) - hpn) * (T(1) - hen), hao = (T(1) - hpo) * (T(1) - heo);
            const T xs = sigmoid_clip(Yv, T(20), T(1e-12));
            const T qd = xs * (T(1) - xs);
            const T ss = ((hgn - hgo) / dt) * (T(c.gpxB) - xs) + ((hpn - hpo) / dt) * (T(1) - xs);
            const T hx = c.prev_level ? hao : han;
            const T gl = (c.gpy == 2 ? hx : (hx > T(c.haeps) ? hx : T(c.haeps))) * qd - T(1);
            src = ss + (c.disable_gamma ? T(0) : gl * dYdt);
        } else if (c.zm) {
            const T th = pf_hp(pn) * ((pp - pn) / dt) * (T(c.vB) - x);
            const T gl = (T(1) - pf_h(pn)) * ld - T(1);
            src = th + gl * dYdt;
        } else {
            const T hn = pf_h(pp), ho = pf_h(pn);
            const T th = T(c.hscale) * ((hn - ho) / dt) * (T(c.vB) - x);
            const T hx = c.prev_level ? ho : hn;
            const T gl = (T(1) - hx) * ld - T(1);
            src = th + (c.disable_gamma ? T(0) : gl * dYdt);
        }
        out[3] = src;
        out[4] = Yf;
    }
    int no_src = 0;   // storage_exact and the splits: the divergence of J alone
    int qmob = 0;     // q split: the matrix-channel mobility
    // GP eta limiter, second flux: the mobility's composition read from this
    // array (the reference's aliased buffer, see gp_y_update), with the FP64
    // thermodynamic constants and Vm_alpha_0, dVm_alpha_dxB, Vm_compound,
    // D_alpha, gp_M_GP, gp_M_beta in md
    const T *xmob = nullptr;
    ThermoConstT<double> tcd{};
    double md[6] = {0, 0, 0, 0, 0, 0};
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        const long long o = row * d.g.NzC + k;
        const T kz = T(d.kt.kz[k]);
        d.S[0][o] = v[0];
        d.S[1][o] = v[1];
        d.S[2][o] = no_src ? cmul_is(v[2], kz) : csub(cmul_is(v[2], kz), v[3]);
        d.S[3][o] = v[4];
    }
};

// (4) y pass: J_x, i ky J_y + (i kz J_z - T), Y^n
template <typename T>
struct OpYCombY {
    static constexpr bool kInplace = false;
    KTab kt;
    __device__ void apply(int, int j, int, const cplx_t<T> *in, cplx_t<T> *out) const {
        out[0] = in[0];
        out[1] = cadd(cmul_is(in[1], T(kt.ky[j])), in[2]);
        out[2] = in[3];
    }
};

// (5) x pass: Y_new_k = mask [Y^n_k + dt (i kx J_x + D) / (1 + dt <DY> k^2)] / N
//   = the reference's Y_semi_implicit_update with rhs_k = divJ_k - T_k
//     - <DY> Lap(Y)_k, Lap(Y)_k = -k^2 Y^n_k (exact algebra, all masks idempotent)
template <typename T>
struct OpYUpdX {
    static constexpr bool kInplace = false;
    KTab kt; double dt, invN; const double *meanDY;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        using T2 = cplx_t<T>;
        if (kt.cut(i, j, k)) { out[0] = mk2<T2>(T(0), T(0)); return; }
        const double den = 1.0 + dt * (*meanDY) * kt.k2(i, j, k);
        const T a = T(dt / den);
        const T2 div = cadd(cmul_is(in[0], T(kt.kx[i])), in[1]);
        out[0] = cscale(cadd(in[2], cscale(div, a)), T(invN));
    }
};

// storage_exact x pass: divJ_k = mask (i kx J_x + i ky J_y + i kz J_z) / N
template <typename T>
struct OpDivX {
    static constexpr bool kInplace = false;
    KTab kt; double invN;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        using T2 = cplx_t<T>;
        if (kt.cut(i, j, k)) { out[0] = mk2<T2>(T(0), T(0)); return; }
        out[0] = cscale(cadd(cmul_is(in[0], T(kt.kx[i])), in[1]), T(invN));
    }
};

// storage_exact final z pass (two_phase_storage_exact_Y_update_kernel,
// cuda_kernels.cu:2859-2921): C^n = (1-h^n) x^n + h^n v_B, the target
// C^n + dt div J, solved for x_alpha with h^{n+1}; where the matrix storage
// 1 - h^{n+1} is below its floor or the solution leaves [eps, 1-eps], x^n
// stays.  Y from the clipped logit, capped at Y_clip.
template <typename T, typename TE>
struct OpStorageExactZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; const cplx_t<T> *src; double ha_eps;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &) const {
        const T Yold = d.Y[cell];
        const T ho = pf_h(clamp01(d.phi_old[cell])), hn = pf_h(clamp01(d.phi_new[cell]));
        const T eps = T(c.xBeps), yc = T(c.Yclip);
        const T xo = sigmoid_clip(Yold + T(d.Yc), yc, eps);
        const T Ct = (T(1) - ho) * xo + ho * T(c.vB) + T(c.dt) * in[0];
        const T han = T(1) - hn;
        const bool small = !(han >= T(ha_eps));
        T xt = xo;
        if (!small && isfinite(Ct)) xt = (Ct - hn * T(c.vB)) / han;
        const bool bad = small || !isfinite(xt) || xt < eps || xt > one_minus_eps(eps);
        const T y = logit_clip(bad ? xo : xt, eps, yc);
        const T yn = y - T(d.Yc);
        d.Y[cell] = yn;
        d.Yprev[cell] = Yold;
        d.dYdt[cell] = (yn - Yold) / T(c.dt);
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
};

// x_transport_projection_split (main_cuda.cu:30564-30676).  z pass: div J
// to real space, the storage source s = div J / (1 - h^{n+1}) where the
// matrix storage reaches its floor, else 0 (compute_xB_storage_rhs_kernel,
// cuda_kernels.cu:2922-2951), and x^n; both forward-transformed
template <typename T, typename TE>
struct OpXSplitSrcZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; double floor_;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = d.S[0][row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *out, Acc &) const {
        const T ha = T(1) - pf_h(clamp01(d.phi_new[cell]));
        out[0] = ha >= T(floor_) ? in[0] / ha : T(0);
        out[1] = sigmoid_clip(d.Y[cell] + T(d.Yc), T(c.Yclip), T(c.xBeps));
    }
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        const long long o = row * d.g.NzC + k;
        d.S[0][o] = v[0];
        d.S[1][o] = v[1];
    }
};

// x pass: the reference's Y_semi_implicit_update_kernel on x with the
// right-hand side S - m Lap(x), m = D_alpha * multiplier:
//   x_k = mask [X_k + dt (S_k + m k^2 X_k)] / (1 + dt m k^2)
//       = mask [X_k + dt S_k / (1 + dt m k^2)]          (exact algebra)
// so the stabiliser damps only the source; / N for the inverse transform
template <typename T>
struct OpXSplitX {
    static constexpr bool kInplace = false;
    KTab kt; double dt, invN, m;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        using T2 = cplx_t<T>;
        if (kt.cut(i, j, k)) { out[0] = mk2<T2>(T(0), T(0)); return; }
        const T a = T(dt / (1.0 + dt * m * kt.k2(i, j, k)));
        out[0] = cscale(cadd(in[1], cscale(in[0], a)), T(invN));
    }
};

// final z pass of the x split (xB_normalize_clamp_and_logit_kernel,
// cuda_kernels.cu:2953-2973): non-finite x keeps x^n, clamp to
// [eps, 1 - eps], Y = logit, capped at +-Y_clip
template <typename T, typename TE>
struct OpXSplitFinalZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; const cplx_t<T> *src;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &) const {
        const T Yold = d.Y[cell];
        const T eps = T(c.xBeps), yc = T(c.Yclip);
        T x = in[0];
        if (!isfinite(x)) x = sigmoid_clip(Yold + T(d.Yc), yc, eps);
        x = fmin(fmax(x, eps), one_minus_eps(eps));
        T y = logit_clip(x, eps, yc);
        y = fmin(fmax(y, -yc), yc);
        const T yn = y - T(d.Yc);
        d.Y[cell] = yn;
        d.Yprev[cell] = Yold;
        d.dYdt[cell] = (yn - Yold) / T(c.dt);
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
};

// ---------------------------------------------------------------------------
// q_transport_projection_split (main_cuda.cu:27781-27783): the matrix storage
// q = (1 - h) x of the conserved composition is the evolved coordinate.
// Tolerances as the reference's calls: feasibility and bound 1e-12.
// ---------------------------------------------------------------------------
constexpr double kQTol = 1.0e-12;

// the bounded context x = q / (1 - h) -> Y (the tail of
// q_normalize_validate_and_reconstruct_kernel and
// q_explicit_transport_and_reconstruct_kernel, cuda_kernels.cu:3032-3105);
// xprev: the current composition, kept where there is no matrix storage
template <typename T, typename PC>
__device__ __forceinline__ T q_context_y(const PC &c, T q, T alpha, T xprev) {
    const T eps = T(c.xBeps), yc = T(c.Yclip);
    T x = alpha > T(1e-14) ? q / alpha : xprev;
    x = fmin(fmax(x, eps), one_minus_eps(eps));
    const T y = logit_clip(x, eps, yc);
    return fmin(fmax(y, -yc), yc);
}

// q = (1 - h) x of the loaded raw fields (initialize_q_alpha_kernel, :2975-2984)
template <typename T>
__global__ void k_q_load(const double *phi, const double *xB, T *q, long long N) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
        q[i] = T((1.0 - pf_h(clamp01(phi[i]))) * xB[i]);
}

// q = (1 - h(phi)) x(Y) (sync_q_from_phi_xB_kernel, :3107-3116; also the
// rebuild after a rejected phase substep).  dydt: the end of the step, where
// dY/dt = (Y - Y^n) / dt is also taken (update_dY_dt_prev_kernel), after a
// redistribution may have moved Y
template <typename T, typename TE>
__global__ void k_q_sync(DevState<T, TE> d, PhysCT<T> c, const T *phi, int dydt) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const T x = sigmoid_clip(d.Y[i] + T(d.Yc), T(c.Yclip), T(c.xBeps));
        d.q[i] = (T(1) - pf_h(clamp01(phi[i]))) * x;
        if (dydt) d.dYdt[i] = (d.Y[i] - d.Yprev[i]) / T(c.dt);
    }
}

// the phase substep's storage transfer q -= (h^{n+1} - h^n) v_B
// (apply_local_phase_storage_transfer_q_kernel, :2989-3019): infeasible cells
// keep q and are counted (block partials); Y of the step's start is kept in
// Yprev for dY/dt
template <typename T, typename TE>
__global__ void k_q_phase(DevState<T, TE> d, PhysCT<T> c) {
    double bad = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        d.Yprev[i] = d.Y[i];
        const T ho = pf_h(clamp01(d.phi_old[i])), hn = pf_h(clamp01(d.phi_new[i]));
        const T an = T(1) - hn;
        const T qn = d.q[i] - (hn - ho) * T(c.vB);
        if (!isfinite(qn) || qn < T(-kQTol) || qn > an + T(kQTol)) { bad += 1.0; continue; }
        d.q[i] = fmin(fmax(qn, T(0)), an);
    }
    AccSum1 s{bad};
    block_reduce_acc(s);
    if (threadIdx.x == 0) reinterpret_cast<AccSum1 *>(d.partials)[blockIdx.x] = s;
}

// q_normalize_validate_and_reconstruct_kernel with invN = 1 (:3032-3069)
template <typename T, typename TE>
__global__ void k_q_reconstruct(DevState<T, TE> d, PhysCT<T> c, const T *phi) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const T alpha = T(1) - pf_h(clamp01(phi[i]));
        T q = d.q[i];
        q = isfinite(q) ? fmin(fmax(q, T(0)), alpha) : T(0);
        d.q[i] = q;
        const T xprev = sigmoid_clip(d.Y[i] + T(d.Yc), T(c.Yclip), T(c.xBeps));
        d.Y[i] = q_context_y<T>(c, q, alpha, xprev) - T(d.Yc);
    }
}

// final z pass of the q split: div J to real space, the explicit transport
// q + dt div J bounded to [0, 1 - h] with the out-of-bounds cells counted
// (q_explicit_transport_and_reconstruct_kernel, :3071-3105), Y from the new
// context, dY/dt against the step's start.  q and div J before the update
// are kept for the local redistribution.
template <typename T, typename TE>
struct OpQTransportZ {
    using Acc = AccSum1;
    DevState<T, TE> d; PhysCT<T> c; const cplx_t<T> *src;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &acc) const {
        const T divJ = in[0];
        const T alpha = T(1) - pf_h(clamp01(d.phi_new[cell]));
        const T q0 = d.q[cell];
        d.qb[cell] = q0;
        d.divr[cell] = divJ;
        const T qt = q0 + T(c.dt) * divJ;
        if (!isfinite(qt) || qt < T(-kQTol) || qt > alpha + T(kQTol)) acc.s += 1.0;
        const T q = isfinite(qt) ? fmin(fmax(qt, T(0)), alpha) : T(0);
        d.q[cell] = q;
        const T xprev = sigmoid_clip(d.Y[cell] + T(d.Yc), T(c.Yclip), T(c.xBeps));
        const T yn = q_context_y<T>(c, q, alpha, xprev) - T(d.Yc);
        d.Y[cell] = yn;
        d.dYdt[cell] = (yn - d.Yprev[cell]) / T(c.dt);
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
    __device__ void finish(int b, const Acc &a) const { reinterpret_cast<Acc *>(d.partials)[b] = a; }
};

// ---------------------------------------------------------------------------
// PF-only conservative composition modes (pf_composition_mode,
// main_cuda.cu:27784-27792; kernels cuda_kernels.cu:3117-3288): the storage
// C = q + h v_B (ctot) or q = (1 - h) x (qalpha) in FP64 on the cell grid,
// moved by limited pairwise face transfers.  FP64 throughout (the storage
// sums must stay conserved); the fields keep their precision.
// ---------------------------------------------------------------------------
// h^-1 by 60 bisections on [0, 1] (h_inverse_bisection_device, :85-97)
__device__ __forceinline__ double h_inverse_bisect(double target) {
    if (target <= 0.0) return 0.0;
    if (target >= 1.0) return 1.0;
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 60; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (pf_h(mid) < target) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

// ---------------------------------------------------------------------------
// GP storage coupling (gp_zone with gp_barrier_only_mode = 0 or
// enable_legacy_gp_storage_coupling = 1): the conserved composition is
// xBtot_gp = h_alpha x + h_GP x_GP + h_beta, with h_beta = h(phi),
// h_GP = (1 - h(phi)) h(eta), h_alpha = (1 - h(phi)) (1 - h(eta))
// (phase_fractions_gp, phase_functions.h:27-42)
// ---------------------------------------------------------------------------
// the matrix composition recovered from a storage target and whether it lies
// in [x_min, x_max] (gp_recovered_xB_valid_device, cuda_kernels.cu:1100-1120)
template <typename T>
__device__ __forceinline__ bool gp_recovered_valid(T tot, T hb, T A, T hg, T xg, T xmin, T xmax, T eh) {
    if (!isfinite(tot) || !isfinite(hb) || !isfinite(A) || !isfinite(hg)) return false;
    if (A < T(0) || hg < T(0) || hg > A) return false;
    const T ha = A - hg;
    if (!(ha >= eh)) return false;
    const T num = tot - hg * xg - hb;
    if (!isfinite(num)) return false;
    const T x = num / ha;
    if (!isfinite(x)) return false;
    return x >= xmin && x <= xmax;
}

// the largest GP fraction in [0, min(h_GP, A)] that keeps the recovered
// composition valid, by 80 bisections (gp_limited_hGP_device, :1122-1149)
template <typename T>
__device__ __forceinline__ T gp_limited_hgp(T tot, T hb, T A, T hg_tent, T xg, T xmin, T xmax, T eh) {
    if (!isfinite(tot) || !isfinite(hb) || !isfinite(A) || !isfinite(hg_tent)) return T(0);
    const T hi0 = fmin(fmax(hg_tent, T(0)), fmax(A, T(0)));
    if (gp_recovered_valid(tot, hb, A, hi0, xg, xmin, xmax, eh)) return hi0;
    T lo = T(0), hi = hi0;
    for (int it = 0; it < 80; ++it) {
        const T mid = T(0.5) * (lo + hi);
        if (gp_recovered_valid(tot, hb, A, mid, xg, xmin, xmax, eh)) lo = mid; else hi = mid;
    }
    return lo;
}

// z pass on div J after the flux (main_cuda.cu:30449-30503): the eta
// feasibility pass (gp_eta_feasibility_and_limiter_kernel, :1151-1250):
// eta^{n+1} clamped to [0, 1]; with the local_clip limiter, where the
// storage target xBtot_gp^n + dt div J admits no matrix composition in
// [xB_eps, 1 - xB_eps] under the tentative GP fraction, the fraction is
// lowered to the largest feasible one and eta follows by inverting h.
// stage 0: the pass alone (the limiter runs it again on a new div J);
// (with keep_div it also keeps div J in divr, the composition of the second
// flux's mobility as the reference computes it);
// stage 1: then the storage point update of Y, gp_storage_exact_Y_update_kernel
// (:2746-2857) or gp_y_picard_iters sweeps of gp_picard_storage_Y_update_kernel
// (:3290-3370) from the guess Y^n; stage 2: then div J kept in divr for the
// right-hand side pass.  Partials: limited cells and <DY> (reduce_sum_DY_gp_kernel,
// :3923-3955, with the final eta).
template <typename T, typename TE>
struct OpGPEtaZ {
    using Acc = AccSum2;
    DevState<T, TE> d; PhysCT<T> c; const cplx_t<T> *src;
    int limiter, stage, picard, iters; double invN;
    int keep_div = 0;   // stage 0: div J kept in divr as well
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &acc) const {
        const T one = T(1), dt = T(c.dt), xg = T(c.gpxB), eh = T(c.haeps);
        const T eps = T(c.xBeps), xmax = one_minus_eps(eps), yc = T(c.Yclip);
        const T dJ = in[0];
        const T Yf = d.Y[cell];
        const T Yn = Yf + T(d.Yc);
        const T pn = d.phi_new[cell], po = d.phi_old[cell], eo = d.eta_old[cell];
        const T et = clamp01(d.eta_new[cell]);
        // feasibility on the clamped fields, x^n the composition of Y^n
        const T xo = sigmoid_clip(Yn, yc, eps);
        const T hpo_c = pf_h(clamp01(po));
        const T hgo_c = (one - hpo_c) * pf_h(clamp01(eo));
        const T hpn_c = pf_h(clamp01(pn));
        const T A = fmax(one - hpn_c, T(0));
        const T hg_tent = A * pf_h(et);
        const T target = (xo + hgo_c * (xg - xo) + hpo_c * (one - xo)) + dt * dJ;
        T ef = et;
        if (limiter && A > eh && hg_tent > T(0) &&
            !gp_recovered_valid(target, hpn_c, A, hg_tent, xg, eps, xmax, eh)) {
            const T hgf = gp_limited_hgp(target, hpn_c, A, hg_tent, xg, eps, xmax, eh);
            const T allowed = clamp01(hgf / fmax(A, eh));
            ef = T(h_inverse_bisect(double(allowed)));
            if (!isfinite(ef)) ef = T(0);
            ef = clamp01(ef);
            if (fabs(et - ef) > T(0)) acc.a += 1.0;
        }
        d.eta_new[cell] = ef;
        if (stage == 0) {
            if (keep_div) d.divr[cell] = dJ;
            return;
        }
        {   // <DY> at phi_for_Y_explicit, eta_for_Y_explicit (main_cuda.cu:30286-30292)
            const T hp = pf_h(c.prev_level ? po : pn), he = pf_h(c.prev_level ? eo : ef);
            const T xs = sigmoid_clip(Yn, T(20), T(1e-12));
            acc.b += double((one - hp) * (one - he) * T(c.Da) * (xs * (one - xs))) * invN;
        }
        if (stage == 2) { d.divr[cell] = dJ; return; }
        // the storage update on the fields as stored (not clamped)
        const T hpo = pf_h(po), heo = pf_h(eo), hpn = pf_h(pn), hen = pf_h(ef);
        const T hgo = (one - hpo) * heo;
        const T hgn = (one - hpn) * hen, han = (one - hpn) * (one - hen);
        const T So = hgo * (xg - xo) + hpo * (one - xo);
        T y;
        if (!picard) {
            const T tot = xo + So + dt * dJ;
            if (!isfinite(tot)) {
                y = Yn;
            } else {
                T xu = xo;
                if (!(han < eh)) xu = (tot - hgn * xg - hpn) / han;
                if (!isfinite(xu)) xu = xo;
                y = logit_clip(xu, eps, yc);
            }
        } else {
            const bool small = han < fmax(eps, T(1.0e-8));
            y = Yn;
            for (int it = 0; it < iters; ++it) {
                const T xs = sigmoid_clip(y, yc, eps);
                T xu = xo;
                if (!small) xu = xo + dt * (dJ - ((hgn * (xg - xs) + hpn * (one - xs)) - So) / dt);
                y = logit_clip(xu, eps, yc);
            }
        }
        const T yn = y - T(d.Yc);
        d.Y[cell] = yn;
        d.Yprev[cell] = Yf;
        d.dYdt[cell] = (yn - Yf) / dt;
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
    __device__ void finish(int b, const Acc &a) const { reinterpret_cast<Acc *>(d.partials)[b] = a; }
};

// R2C z pass of the limited-eta right-hand side: R = div J - S - gamma dY/dt
// from the div J kept by OpGPEtaZ (compute_Y_rhs_gp_kernel :2361-2430 /
// compute_Y_rhs_gp_conservative_kernel :2432-2527 less the Laplacian term,
// which the x pass applies), and Y^n
template <typename T, typename TE>
struct OpGPRhsZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c;
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void point(long long cell, const T *, T *out, Acc &) const {
        const T one = T(1), dt = T(c.dt);
        const T Yf = d.Y[cell];
        const T pn = d.phi_new[cell], po = d.phi_old[cell];
        const T hpn = pf_h(pn), hen = pf_h(d.eta_new[cell]), hpo = pf_h(po), heo = pf_h(d.eta_old[cell]);
        const T hgn = (one - hpn) * hen, hgo = (one - hpo) * heo;
        const T han = (one - hpn) * (one - hen), hao = (one - hpo) * (one - heo);
        const T xs = sigmoid_clip(Yf + T(d.Yc), T(20), T(1e-12));
        const T ss = ((hgn - hgo) / dt) * (T(c.gpxB) - xs) + ((hpn - hpo) / dt) * (one - xs);
        const T hx = c.prev_level ? hao : han;
        const T gl = (c.gpy == 2 ? hx : (hx > T(c.haeps) ? hx : T(c.haeps))) * (xs * (one - xs)) - one;
        const T dYdt = d.dYdt[cell] + T(d.dYoff);
        out[0] = d.divr[cell] - ss - (c.disable_gamma ? T(0) : gl * dYdt);
        out[1] = Yf;
    }
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        const long long o = row * d.g.NzC + k;
        d.S[0][o] = v[0];
        d.S[1][o] = v[1];
    }
};

// x pass of that update: Y_k = mask [Y^n_k + dt R_k / (1 + dt <DY> k^2)] / N
// (Y_semi_implicit_update_kernel with rhs = R - <DY> Lap Y^n, exact algebra)
template <typename T>
struct OpYUpdRX {
    static constexpr bool kInplace = false;
    KTab kt; double dt, invN; const double *meanDY;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        using T2 = cplx_t<T>;
        if (kt.cut(i, j, k)) { out[0] = mk2<T2>(T(0), T(0)); return; }
        const T a = T(dt / (1.0 + dt * (*meanDY) * kt.k2(i, j, k)));
        out[0] = cscale(cadd(in[1], cscale(in[0], a)), T(invN));
    }
};

// x from the storage, the equilibrium composition where the matrix vanishes
// or x is not finite, bounded; its logit (the shared tail of
// reconstruct_conservative_context_kernel and
// constrain_phase_and_reconstruct_conservative_kernel)
__device__ __forceinline__ double cons_y(double q, double alpha, double beta_eps, double xeq, double eps,
                                        double yclip, bool *nonfinite) {
    double x = xeq;
    if (alpha > beta_eps) x = q / alpha;
    if (!isfinite(x)) { x = xeq; *nonfinite = true; }
    x = fmin(fmax(x, eps), 1.0 - eps);
    return logit_clip(x, eps, yclip);
}

struct ConsArgs {
    int ctot, be;
    double vB, beta_eps, xeq, eps, yclip, tol, dt, Da;
};
static ConsArgs cons_args(const pfgb_ctx *c) {
    const pfgb_params &P = c->p;
    ConsArgs a;
    a.ctot = P.pf_composition_mode == PFGB_COMPOSITION_CTOT;
    a.be = P.pf_conservative_flux_strategy == PFGB_CONS_FLUX_BACKWARD_EULER;
    a.vB = P.v_B;
    a.beta_eps = P.pf_conservative_beta_support_eps;
    a.xeq = P.xB_eq_matrix;
    a.eps = P.xB_eps;
    a.yclip = P.Y_clip;
    a.tol = P.pf_conservative_bound_tol;
    a.dt = P.dt;
    a.Da = P.D_alpha;
    return a;
}

// initialize_conservative_storage_kernel (:3123-3132), from the loaded fields
__global__ void k_cons_load(const double *phi, const double *xB, double *cst, long long N, int ctot, double vB) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const double h = pf_h(clamp01(phi[i]));
        const double q = (1.0 - h) * clamp01(xB[i]);
        cst[i] = ctot ? q + h * vB : q;
    }
}

// reconstruct_conservative_context_kernel (:3134-3159) at phi
template <typename T, typename TE>
__global__ void k_cons_context(DevState<T, TE> d, ConsArgs a, const double *cst, const T *phi) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const double h = pf_h(clamp01(double(phi[i])));
        const double alpha = fmax(1.0 - h, 0.0);
        const double q = a.ctot ? cst[i] - h * a.vB : cst[i];
        bool nf = false;
        d.Y[i] = T(cons_y(q, alpha, a.beta_eps, a.xeq, a.eps, a.yclip, &nf) - d.Yc);
    }
}

// compute_mu_x_kernel (:1266-1324) at phi^n in real space, FP64, with the
// stress stored by the last elastic solve
template <typename T, typename TE>
__global__ void k_cons_mu(DevState<T, TE> d, PhysC c, double *mu) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const double xB = sigmoid_clip(double(d.Y[i]) + d.Yc, c.Yclip, c.xBeps);
        double offA, offB;
        thermo_mu_off<double>(c.tc, xB, offA, offB);
        const double h = pf_h(double(d.phi_old[i]));
        const double cb = c_xB_phi<double>(xB, c.Vm0, c.dVm, c.Vmc, h);
        const double muA = c.tc.GA_s + offA, muB = c.tc.GB_s + offB;
        const double mt = (1.0 - h) * (muA * (1.0 - xB) + muB * xB) + h * c.mu0;
        double m = cb * ((c.dG + offB - offA) - cb * mt * c.dVm);
        if (c.elastic && d.sig[0]) m += -c.eiv * (double(d.sig[0][i]) + double(d.sig[1][i]) + double(d.sig[2][i]));
        mu[i] = m;
    }
}

// one checkerboard sweep of the pairwise face transfer
// (pairwise_conservative_face_sweep_kernel, :3161-3237): the face between
// each cell of the given coordinate parity and its + neighbour (periodic);
// mobilities (1 - h) M_alpha joined harmonically; dt M (mu_i - mu_j) / dx^2,
// damped in the backward-Euler strategy; limited by both cells' storage
// bounds.  Every cell lies on one face of a sweep, so the faces run in
// parallel.  The limited faces are counted (block partials).
template <typename T, typename TE>
__global__ void k_cons_sweep(DevState<T, TE> d, PhysC c, ConsArgs a, double *cst, const double *mu, int axis,
                             int parity, double spacing) {
    double lim = 0.0;
    const int Nx = d.g.Nx, Ny = d.g.Ny, Nz = d.g.Nz;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < d.g.N;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx % Nz), t = (int)(idx / Nz), j = t % Ny, i = t / Ny;
        const int coord = axis == 0 ? i : (axis == 1 ? j : k);
        if ((coord & 1) != parity) continue;
        int ni = i, nj = j, nk = k;
        if (axis == 0) ni = i + 1 == Nx ? 0 : i + 1;
        else if (axis == 1) nj = j + 1 == Ny ? 0 : j + 1;
        else nk = k + 1 == Nz ? 0 : k + 1;
        const long long n = ((long long)ni * Ny + nj) * Nz + nk;
        const double hi = pf_h(clamp01(double(d.phi_old[idx]))), hj = pf_h(clamp01(double(d.phi_old[n])));
        const double ai = fmax(1.0 - hi, 0.0), aj = fmax(1.0 - hj, 0.0);
        const double xi = fmin(fmax(sigmoid_clip(double(d.Y[idx]) + d.Yc, c.Yclip, c.xBeps), 1e-12), 1.0 - 1e-12);
        const double xj = fmin(fmax(sigmoid_clip(double(d.Y[n]) + d.Yc, c.Yclip, c.xBeps), 1e-12), 1.0 - 1e-12);
        const double Gi = gamma_thermo<double>(c.tc, xi, 0.0, c.Vm0, c.dVm, c.Vmc);
        const double Gj = gamma_thermo<double>(c.tc, xj, 0.0, c.Vm0, c.dVm, c.Vmc);
        const double Mi = ai * stabilized_meff<double>(a.Da, Gi), Mj = aj * stabilized_meff<double>(a.Da, Gj);
        const double Mf = (Mi > 0.0 && Mj > 0.0) ? 2.0 * Mi * Mj / (Mi + Mj) : 0.0;
        const double inv2 = 1.0 / (spacing * spacing);
        double tr = a.dt * Mf * (mu[idx] - mu[n]) * inv2;
        if (a.be && Mf > 0.0) {
            const double di = Gi / fmax(ai, 1.0e-14), dj = Gj / fmax(aj, 1.0e-14);
            tr /= 1.0 + a.dt * Mf * inv2 * fmax(di + dj, 0.0);
        }
        const double si = cst[idx], sj = cst[n];
        const double loi = a.ctot ? hi * a.vB : 0.0, loj = a.ctot ? hj * a.vB : 0.0;
        const double upi = a.ctot ? hi * a.vB + ai : ai, upj = a.ctot ? hj * a.vB + aj : aj;
        const double raw = tr;
        if (tr >= 0.0) {
            tr = fmin(tr, fmax(si - loi, 0.0));
            tr = fmin(tr, fmax(upj - sj, 0.0));
        } else {
            const double mag = fmin(-tr, fmax(sj - loj, 0.0));
            tr = -fmin(mag, fmax(upi - si, 0.0));
        }
        if (fabs(tr - raw) > a.tol) lim += 1.0;
        cst[idx] = si - tr;
        cst[n] = sj + tr;
    }
    AccSum1 s{lim};
    block_reduce_acc(s);
    if (threadIdx.x == 0) reinterpret_cast<AccSum1 *>(d.partials)[blockIdx.x] = s;
}

// constrain_phase_and_reconstruct_conservative_kernel (:3239-3288) on the
// new phi: h capped at C / v_B (phi by bisection); a cell whose storage would
// leave its bounds keeps phi^n (counted: the step is rejected); qalpha stores
// q for the new h; the context.  Partials: rejected and capped cells.
template <typename T, typename TE>
__global__ void k_cons_constrain(DevState<T, TE> d, ConsArgs a, double *cst) {
    double bad = 0.0, capped = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const double po = clamp01(double(d.phi_old[i]));
        const double ho = pf_h(po);
        const double C = a.ctot ? cst[i] : cst[i] + ho * a.vB;
        double phi = clamp01(double(d.phi_new[i]));
        double h = pf_h(phi);
        const double hmax = a.vB > 0.0 ? fmin(fmax(C / a.vB, 0.0), 1.0) : 1.0;
        if (h > hmax + a.tol) {
            phi = h_inverse_bisect(hmax);
            h = pf_h(phi);
            capped += 1.0;
        }
        double alpha = fmax(1.0 - h, 0.0);
        double q = C - h * a.vB;
        if (!isfinite(q) || q < -a.tol || q > alpha + a.tol) {
            bad += 1.0;
            phi = po;
            h = ho;
            alpha = fmax(1.0 - h, 0.0);
            q = C - h * a.vB;
        }
        d.phi_new[i] = T(phi);
        if (!a.ctot) cst[i] = q;
        bool nf = false;
        d.Y[i] = T(cons_y(q, alpha, a.beta_eps, a.xeq, a.eps, a.yclip, &nf) - d.Yc);
        if (nf) bad += 1.0;
    }
    AccSum2 s{bad, capped};
    block_reduce_acc(s);
    if (threadIdx.x == 0) reinterpret_cast<AccSum2 *>(d.partials)[blockIdx.x] = s;
}

// (6) final z pass: store Y_f, dY/dt, and the zero-mode statistics
template <typename T, typename TE>
struct OpYFinalZ {
    using Acc = AccZMt<T>;
    DevState<T, TE> d; PhysCT<T> c; const cplx_t<T> *src;
    // Y^n (and phi^{n+1} for the moments) of eight cells read ahead of their stores
    static constexpr int kBatch = 8;
    struct Pre { T Y, phin; };
    __device__ void fetch(long long cell, Pre &p) const {
        p.Y = d.Y[cell];
        p.phin = c.zm ? d.phi_new[cell] : T(0);
    }
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *out, Acc &acc) const {
        Pre p;
        fetch(cell, p);
        point_with(cell, p, in, out, acc);
    }
    __device__ void point_with(long long cell, const Pre &p, const T *in, T *, Acc &acc) const {
        const T Yold = p.Y;
        T y = in[0];
        if (!c.zm) {
            // Y_normalize_and_clamp_kernel (:2554-2572), Y_cap = Y_clip, with
            // the bounds moved to the stored frame (no round trip through Y + Yc)
            const T hi = T(c.Yclip - d.Yc), lo = T(-c.Yclip - d.Yc);
            if (y > hi) y = hi;
            if (y < lo) y = lo;
        }
        d.Y[cell] = y;
        d.Yprev[cell] = Yold;
        d.dYdt[cell] = (y - Yold) / T(c.dt);
        if (c.zm) {
            // min / max of the stored Y* (exact: the offset Yc is added after
            // the reduction); the Taylor moments feed only the Newton
            // predictor and sum|1-h| only a bound, so field precision is enough
            acc.mn = fmin(acc.mn, y);
            acc.mx = fmax(acc.mx, y);
            const T h = pf_h(p.phin);
            const T a = T(1) - h;
            const T s = sigmoid_raw(y + T(d.Yc));
            const T s1 = s * (T(1) - s);
            const T u = T(1) - T(2) * s;
            acc.m[0] += a * s + h * T(c.vB);
            acc.m[1] += a * s1;
            acc.m[2] += a * s1 * u;
            acc.m[3] += a * s1 * (T(1) - T(6) * s1);
            acc.m[4] += a * s1 * u * (T(1) - T(12) * s1);
            acc.m[5] += fabs(a);
        }
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
    __device__ void finish(int b, const Acc &a) const {
        AccZM w;
        w.mn = double(a.mn);
        w.mx = double(a.mx);
#pragma unroll
        for (int i = 0; i < 6; ++i) w.m[i] = double(a.m[i]);
        reinterpret_cast<AccZM *>(d.partials)[b] = w;
    }
};

// zero-mode direct evaluation: mass(l) and d mass/dl at given shifts, FP64
// (compute_pf_Y_zero_mode_terms_kernel, cuda_kernels.cu:3409-3420).  nl shifts
// at once; used for the bracket ends and when the Taylor model is out of range.
// TV = evaluation precision: double for every convergence decision; the
// field precision for the bracket-end check, whose margin is then verified
// mass and its derivative at NL trial multipliers (NL = 1 or 2; compile
// time, so the sums stay in registers).  sigmoid(y + lam) is evaluated as
// 1 / (1 + e^-y e^-lam): one exponential per cell, e^-lam once per thread.
// Cells with |y| beyond half the exponent range of TV (where e^-y could
// overflow) take sigmoid(y + lam) directly.
template <typename T, typename TV, int NL>
__global__ void k_zm_eval(const T *Y, const T *phi, long long N, double Yc, double vB,
                          const double *lam, double *partials) {
    constexpr double kBig = sizeof(TV) == 4 ? 40.0 : 300.0;
    double m[NL], dd[NL], lv[NL];
    TV el[NL];
#pragma unroll
    for (int q = 0; q < NL; ++q) {
        m[q] = 0.0; dd[q] = 0.0; lv[q] = lam[q];
        el[q] = fabs(lv[q]) < kBig ? exp(TV(-lv[q])) : TV(0);
    }
    // sums in TV over chunks of 16 cells of a thread, then into FP64: the
    // FP32 evaluation (bracket decisions with a 1e-5 relative margin) no
    // longer spends the FP64 pipe on every cell
    TV cm[NL], cd[NL];
#pragma unroll
    for (int q = 0; q < NL; ++q) { cm[q] = TV(0); cd[q] = TV(0); }
    int cnt = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const TV h = pf_h(TV(phi[i]));
        const TV a = TV(1) - h;
        const double y = double(Y[i]) + Yc;
        const TV ey = exp(TV(-y));
        const TV hv = h * TV(vB);
#pragma unroll
        for (int q = 0; q < NL; ++q) {
            const TV x = (fabs(y) < kBig && fabs(lv[q]) < kBig) ? TV(1) / (TV(1) + ey * el[q])
                                                               : sigmoid_raw(TV(y + lv[q]));
            cm[q] += a * x + hv;
            cd[q] += a * x * (TV(1) - x);
        }
        if (++cnt == (sizeof(TV) == 4 ? 16 : 1)) {
#pragma unroll
            for (int q = 0; q < NL; ++q) { m[q] += double(cm[q]); dd[q] += double(cd[q]); cm[q] = TV(0); cd[q] = TV(0); }
            cnt = 0;
        }
    }
#pragma unroll
    for (int q = 0; q < NL; ++q) { m[q] += double(cm[q]); dd[q] += double(cd[q]); }
#pragma unroll
    for (int q = 0; q < NL; ++q) {
        AccSum2 s{m[q], dd[q]};
        block_reduce_acc(s);
        if (threadIdx.x == 0) reinterpret_cast<AccSum2 *>(partials)[q * gridDim.x + blockIdx.x] = s;
        __syncthreads();
    }
}

// The exact evaluation of the FP32-field path in double-float arithmetic
// (dfloat.cuh): per cell h(phi), 1 - h, sigmoid(Y* + Yc + l) and the mass
// term (1 - h) s + h v_B on the FP32 pipe, summed in double-float over
// chunks of 16 cells of a thread, the chunks in FP64 and the blocks in FP64.
// A cell's term carries a relative error of a few 2^-48 and the chunk sums
// about 2^-44, so the total stays within about 1e-13 relative of the FP64
// evaluation (k_zm_eval<T, double>), under the 1e-12 the mass ledger holds.
// The derivative feeds only the Newton steps and is summed in float chunks.
template <int NL>
__global__ void k_zm_eval_df(const float *Y, const float *phi, long long N, double Yc, double vB,
                             const double *lam, double *partials) {
    __shared__ float2 tab[64];
    if (threadIdx.x < 64) tab[threadIdx.x] = dfexp::kExp2Tab[threadIdx.x];
    __syncthreads();
    dfl c[NL], cm[NL];
    double m[NL], dd[NL];
    float cd[NL];
#pragma unroll
    for (int q = 0; q < NL; ++q) {
        c[q] = df_from_double(Yc + lam[q]);
        cm[q] = dfl{0.f, 0.f};
        m[q] = 0.0; dd[q] = 0.0; cd[q] = 0.f;
    }
    const dfl vb = df_from_double(vB);
    int cnt = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const float p = phi[i];
        // h = p^3 (10 + p (6 p - 15)), p exact
        dfl t = df_add_f(df_two_prod(6.0f, p), -15.0f);
        t = df_add_f(df_mul_f(t, p), 10.0f);
        const dfl h = df_mul(df_mul_f(df_two_prod(p, p), p), t);
        const dfl a = df_add_f(df_neg(h), 1.0f);
        const dfl hv = df_mul(h, vb);
        const float y = Y[i];
#pragma unroll
        for (int q = 0; q < NL; ++q) {
            const dfl sg = df_sigmoid(df_add_f(c[q], y), tab);
            cm[q] = df_add(cm[q], df_add(df_mul(a, sg), hv));
            cd[q] = fmaf(a.hi * sg.hi, 1.0f - sg.hi, cd[q]);
        }
        if (++cnt == 16) {
#pragma unroll
            for (int q = 0; q < NL; ++q) {
                m[q] += df_to_double(cm[q]); dd[q] += (double)cd[q];
                cm[q] = dfl{0.f, 0.f}; cd[q] = 0.f;
            }
            cnt = 0;
        }
    }
#pragma unroll
    for (int q = 0; q < NL; ++q) { m[q] += df_to_double(cm[q]); dd[q] += (double)cd[q]; }
#pragma unroll
    for (int q = 0; q < NL; ++q) {
        AccSum2 s{m[q], dd[q]};
        block_reduce_acc(s);
        if (threadIdx.x == 0) reinterpret_cast<AccSum2 *>(partials)[q * gridDim.x + blockIdx.x] = s;
        __syncthreads();
    }
}

// ===========================================================================
// Elastic solve
// ===========================================================================
// cold start producer: eigenstrain eps0 -> R2C (6 fields)
template <typename T, typename TE>
struct OpEigenR2C {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec;
    __device__ void point(long long cell, const TE *, TE *out, Acc &) const {
        const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
        eigenstrain<T, TE>(c, ec, d.phi_old[cell], c.gp ? d.eta_old[cell] : T(0), xB_el(c, xB),
                           c.gp_el != 0, out);
    }
    __device__ void load_spec(long long, int, cplx_t<TE> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<TE> *v) const {
        const long long o = row * d.g.NzC + k;
#pragma unroll
        for (int a = 0; a < 6; ++a) d.E[a][o] = v[a];
    }
};

// iteration: C2R strain (/N) -> h = C0:eps - (C0 + h dC):(eps + E0 - eps0)
// (compute_strain_with_perturbation_kernel, cuda_kernels.cu:7002-7157) -> R2C
template <typename T, typename TE>
struct OpHijZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec;
    int lin;   // increment form: the linear part -(h dC):eps only
    __device__ void load_spec(long long row, int k, cplx_t<TE> *v) const {
        const long long o = row * d.g.NzC + k;
#pragma unroll
        for (int a = 0; a < 6; ++a) v[a] = d.E[a][o];
    }
    __device__ void point(long long cell, const TE *in, TE *out, Acc &) const {
        TE e[6], e0[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) e[a] = in[a] * ec.invN;
        const T phi = d.phi_old[cell];
        const T h = pf_h(phi);
        TE tv[6];
        if (lin) {
#pragma unroll
            for (int a = 0; a < 6; ++a) tv[a] = e[a];
        } else {
            const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
            eigenstrain<T, TE>(c, ec, phi, c.gp ? d.eta_old[cell] : T(0), xB_el(c, xB), c.gp_el != 0, e0);
#pragma unroll
            for (int a = 0; a < 6; ++a) tv[a] = e[a] + ec.E0[a] - e0[a];
        }
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            TE acc = 0;
#pragma unroll
            for (int b = 0; b < 6; ++b) {
                const int v = vidx(a, b);
                const TE c0 = ec.S[v];
                const TE ce = c0 + (TE)(h * T(ec.Sp[v]));
                const TE f = b >= 3 ? TE(2) : TE(1);
                acc += f * (c0 * e[b] - ce * tv[b]);
            }
            out[a] = acc;
        }
    }
    __device__ void store_spec(long long row, int k, const cplx_t<TE> *v) const {
        const long long o = row * d.g.NzC + k;
#pragma unroll
        for (int a = 0; a < 6; ++a) d.E[a][o] = v[a];
    }
};

// finalize: C2R strain, /N, + E0 -> stored total strain
template <typename T, typename TE>
struct OpStrainFinalZ {
    using Acc = NoAcc;
    DevState<T, TE> d; ElasC<TE> ec; PhysCT<T> c;
    __device__ void load_spec(long long row, int k, cplx_t<TE> *v) const {
        const long long o = row * d.g.NzC + k;
#pragma unroll
        for (int a = 0; a < 6; ++a) v[a] = d.E[a][o];
    }
    __device__ void point(long long cell, const TE *in, TE *, Acc &) const {
        TE e[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) {
            e[a] = in[a] * ec.invN + ec.E0[a];
            d.eps[a][cell] = e[a];
        }
        if (d.sig[0]) {
            // compute_stress_from_strain_with_effective_stiffness_kernel
            // (:7381-7480): the stress kept for the rest of the iteration
            TE sg[6];
            const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
            stress_at<T, TE>(c, ec, d.phi_old[cell], c.gp ? d.eta_old[cell] : T(0), xB, e, sg);
#pragma unroll
            for (int a = 0; a < 6; ++a) d.sig[a][cell] = sg[a];
        }
    }
    __device__ void store_spec(long long, int, const cplx_t<TE> *) const {}
};

// symmetric strain of a displacement: eps_ab = i (k_a u_b + k_b u_a) / 2
// (compute_strain_from_displacement_k_kernel, cuda_kernels.cu:6673-6730)
template <typename TE>
__device__ __forceinline__ cplx_t<TE> strain_comp(int comp, TE kx, TE ky, TE kz, const cplx_t<TE> *u) {
    const TE kv[3] = {kx, ky, kz};
    const int a = comp < 3 ? comp : (comp == 3 ? 1 : 0);
    const int b = comp < 3 ? comp : (comp == 5 ? 1 : 2);
    if (a == b) return cmul_is(u[a], kv[a]);
    const cplx_t<TE> s = cadd(cscale(u[b], kv[a]), cscale(u[a], kv[b]));
    return cmul_is(s, TE(0.5));
}

template <typename TE>
struct OpStrainFromUX {   // warm start: strain of the stored u, then inverse x
    static constexpr bool kInplace = false;
    KTab kt;
    __device__ void apply(int i, int j, int k, const cplx_t<TE> *u, cplx_t<TE> *out) const {
        const TE kx = TE(kt.kx[i]), ky = TE(kt.ky[j]), kz = TE(kt.kz[k]);
        const bool m = kt.cut(i, j, k);
#pragma unroll
        for (int cmp = 0; cmp < 6; ++cmp)
            out[cmp] = m ? mk2<cplx_t<TE>>(TE(0), TE(0)) : strain_comp<TE>(cmp, kx, ky, kz, u);
    }
};

// Green's function x pass.  Inputs: the 6 y-transformed components of the
// source (eps0 for the cold start, h_ij during the iteration).
//   t_i = k_j tau_ij  (tau = C0:eps0 for EIGEN)
//   u   = -i G(k) t,  G = K^-1, K_ij = k_a C_iajb k_b, u(k=0) = 0, dealiased
//   (compute_displacement_from_eigenstrain_k_kernel :6734-6998,
//    compute_displacement_from_hij_green_kernel :6484-6634)
// The new u is stored (warm state), the Hermitian-weighted residual against
// the previous u is accumulated (compute_elastic_displacement_residual_kernel
// :6436-6467), and the 6 strain components of u are inverse x transformed.
template <typename TE>
struct GreenArgs {
    Grid3 g; KTab kt; ElasC<TE> ec;
    const cplx_t<TE> *tw;
    cplx_t<TE> *E[6], *U[3];
    cplx_t<TE> *R[3], *D[3];   // increment form: r0 and delta
    cplx_t<TE> *Dm[3];         // Chebyshev: the iterate before delta (null: plain update)
    TE gam, rho;
    double *partials;
    const double *skip;        // return at once when *skip != 0 (a finished solve)
    const float4 *btab;        // tensor-core 41-point stage: its B table (null: FP32 FMAs)
    int *tc_err;               // set when a bounded tensor-core wait runs out
    int resid;
    int mode;                  // 0 u <- Phi(u); 1 first increment step; 2 delta <- r0 + L delta
};

// the Green's-operator output at one k-point, by update form: stores the new
// state, accumulates the residual sums, and returns the field whose strain
// goes on (u, or the increment delta)
template <typename TE>
__device__ __forceinline__ void green_update(const GreenArgs<TE> &A, long long o, const cplx_t<TE> u[3], TE w,
                                             TE &rd, TE &rr, cplx_t<TE> out[3]) {
    using T2 = cplx_t<TE>;
    TE ld_ = 0, lr = 0;
    if (A.mode == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if (A.resid) {
                const T2 old = A.U[c][o];
                const TE dr = u[c].x - old.x, di = u[c].y - old.y;
                ld_ += dr * dr + di * di;
                lr += u[c].x * u[c].x + u[c].y * u[c].y;
            }
            A.U[c][o] = u[c];
            out[c] = u[c];
        }
    } else if (A.mode == 1) {
        // r0 = u1 - u0; delta_1 = r0 (Chebyshev: the relaxed gam r0, with the
        // iterate before it, delta_0 = 0)
        const bool cheb = A.Dm[0] != nullptr;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T2 u0 = A.U[c][o];
            const T2 r = mk2<T2>(u[c].x - u0.x, u[c].y - u0.y);
            A.R[c][o] = r;
            const T2 x1 = cheb ? mk2<T2>(A.gam * r.x, A.gam * r.y) : r;
            A.D[c][o] = x1;
            if (cheb) A.Dm[c][o] = mk2<T2>(TE(0), TE(0));
            ld_ += r.x * r.x + r.y * r.y;
            lr += u[c].x * u[c].x + u[c].y * u[c].y;
            out[c] = x1;
        }
    } else {
        // g = r0 + L delta; the residual |g - delta| / |u0 + g| is the
        // reference's |u_new - u_old| / |u_new| for a plain step from delta.
        // Plain: delta <- g.  Chebyshev: y = delta + gam (g - delta),
        // delta_new = delta_prev + rho (y - delta_prev), written over delta_prev
        // (the host swaps the two buffers).
        const bool cheb = A.Dm[0] != nullptr;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T2 r0 = A.R[c][o], d = A.D[c][o], u0 = A.U[c][o];
            const T2 dn = mk2<T2>(r0.x + u[c].x, r0.y + u[c].y);
            const TE dr = dn.x - d.x, di = dn.y - d.y;
            const TE ur = u0.x + dn.x, ui = u0.y + dn.y;
            ld_ += dr * dr + di * di;
            lr += ur * ur + ui * ui;
            if (cheb) {
                const T2 xm = A.Dm[c][o];
                const TE yr = d.x + A.gam * dr, yi = d.y + A.gam * di;
                const T2 xn = mk2<T2>(xm.x + A.rho * (yr - xm.x), xm.y + A.rho * (yi - xm.y));
                A.Dm[c][o] = xn;
                out[c] = xn;
            } else {
                A.D[c][o] = dn;
                out[c] = dn;
            }
        }
    }
    rd += w * ld_;
    rr += w * lr;
}

// the state the increment update (mode 2) reads at one k-point, loaded as
// one batch ahead of use: r0, delta, u0 and the Chebyshev iterate before delta
template <typename TE>
struct GreenIn { cplx_t<TE> r0[3], d[3], u0[3], dm[3]; };

template <typename TE>
__device__ __forceinline__ void green_fetch(const GreenArgs<TE> &A, long long o, GreenIn<TE> &in) {
    const bool cheb = A.Dm[0] != nullptr;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        in.r0[c] = __ldg(A.R[c] + o);
        in.d[c] = __ldg(A.D[c] + o);
        in.u0[c] = __ldg(A.U[c] + o);
        in.dm[c] = cheb ? A.Dm[c][o] : cplx_t<TE>{};
    }
}

// green_update's mode 2 on prefetched state; the stores go last
template <typename TE>
__device__ __forceinline__ void green_update_in(const GreenArgs<TE> &A, long long o, const GreenIn<TE> &in,
                                                const cplx_t<TE> u[3], TE w, TE &rd, TE &rr, cplx_t<TE> out[3]) {
    using T2 = cplx_t<TE>;
    const bool cheb = A.Dm[0] != nullptr;
    TE ld_ = 0, lr = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T2 dn = mk2<T2>(in.r0[c].x + u[c].x, in.r0[c].y + u[c].y);
        const TE dr = dn.x - in.d[c].x, di = dn.y - in.d[c].y;
        const TE ur = in.u0[c].x + dn.x, ui = in.u0[c].y + dn.y;
        ld_ += dr * dr + di * di;
        lr += ur * ur + ui * ui;
        if (cheb) {
            const T2 xm = in.dm[c];
            const TE yr = in.d[c].x + A.gam * dr, yi = in.d[c].y + A.gam * di;
            out[c] = mk2<T2>(xm.x + A.rho * (yr - xm.x), xm.y + A.rho * (yi - xm.y));
        } else {
            out[c] = dn;
        }
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) (cheb ? A.Dm[c] : A.D[c])[o] = out[c];
    rd += w * ld_;
    rr += w * lr;
}

template <typename TE>
__device__ __forceinline__ void green_u(const TE *S, TE kx, TE ky, TE kz, const cplx_t<TE> t[3],
                                        cplx_t<TE> u[3]) {
    const TE kv[3] = {kx, ky, kz};
    TE K[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
            TE acc = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) acc += kv[a] * S[vidx(tvoigt(i, a), tvoigt(j, b))] * kv[b];
            K[i][j] = acc;
            K[j][i] = acc;
        }
    const TE c00 = K[1][1] * K[2][2] - K[1][2] * K[1][2];
    const TE c01 = K[0][2] * K[1][2] - K[0][1] * K[2][2];
    const TE c02 = K[0][1] * K[1][2] - K[0][2] * K[1][1];
    const TE c11 = K[0][0] * K[2][2] - K[0][2] * K[0][2];
    const TE c12 = K[0][2] * K[0][1] - K[0][0] * K[1][2];
    const TE c22 = K[0][0] * K[1][1] - K[0][1] * K[0][1];
    const TE det = K[0][0] * c00 + K[0][1] * c01 + K[0][2] * c02;
    using T2 = cplx_t<TE>;
    if (fabs((double)det) < 1e-30) { u[0] = u[1] = u[2] = mk2<T2>(TE(0), TE(0)); return; }
    const TE id = TE(1) / det;
    const TE G[3][3] = {{c00 * id, c01 * id, c02 * id}, {c01 * id, c11 * id, c12 * id}, {c02 * id, c12 * id, c22 * id}};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T2 s = mk2<T2>(TE(0), TE(0));
#pragma unroll
        for (int b = 0; b < 3; ++b) s = cadd(s, cscale(t[b], G[a][b]));
        u[a] = mk2<T2>(s.y, -s.x);   // -i s
    }
}

template <typename TE, bool EIGEN>
__global__ void __launch_bounds__(256)
k_x_green(GreenArgs<TE> A, AxisPlan plan, int TK) {
    if (A.skip && *A.skip != 0.0) return;
    using T2 = cplx_t<TE>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *sm = reinterpret_cast<T2 *>(smem_raw);
    const int n = plan.n, SP = 6 * TK + 1;   // six components interleaved per row
    T2 *tw = sm;
    T2 *X = sm + n, *Yb = X + n * SP;
    const int k0 = blockIdx.x * TK, j = blockIdx.y;
    const long long base = (long long)j * A.g.NzC + k0;
    const long long es = (long long)A.g.Ny * A.g.NzC;
    const int kcnt = min(TK, A.g.NzC - k0);
    const int lgTK = __ffs(TK) - 1;
#pragma unroll
    for (int cmp = 0; cmp < 6; ++cmp) {
        for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
            const int q = e >> lgTK, l = e & (TK - 1);
            const bool ok = l < kcnt;
            cp_async_elem(&X[q * SP + cmp * TK + l], A.E[cmp] + (ok ? base + q * es + l : base), ok);
        }
    }
    cp_async_commit();
    load_tw<TE>(tw, A.tw, n);
    cp_async_wait_all();
    __syncthreads();
    T2 *cur = fft_lines<TE, -1>(X, Yb, plan, tw, 6 * TK, SP, 1, false);
    T2 *oth = (cur == X) ? Yb : X;
    // per point: t_i = k_j tau_ij, u = -i G t (masked), residual, u stored,
    // then the six strain components of u into the other buffer
    // residual sums: per element in elastic precision, per-thread partials
    // (a handful of elements) in elastic precision, block / grid sums in FP64
    TE rd = 0, rr = 0;
    const bool pre = A.mode == 2;   // increment update: its state loaded as one batch first
    for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
        const int q = e >> lgTK, l = e & (TK - 1), k = k0 + l;
        GreenIn<TE> gin;
        if (pre && l < kcnt) green_fetch<TE>(A, base + q * es + l, gin);
        const int kk = min(k, A.g.NzC - 1);
        const TE kv[3] = {TE(A.kt.kx[q]), TE(A.kt.ky[j]), TE(A.kt.kz[kk])};
        T2 x[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) x[c] = cur[q * SP + c * TK + l];
        T2 t[3];
        if (EIGEN) {
            // tau_ij = C_ij,ab eps0_ab: component c enters with weight 1
            // (normal) or 2 (shear) in Voigt column c
#pragma unroll
            for (int ii = 0; ii < 3; ++ii) {
                T2 acc = mk2<T2>(TE(0), TE(0));
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    TE s = 0;
#pragma unroll
                    for (int jj = 0; jj < 3; ++jj) s += kv[jj] * A.ec.S[vidx(tvoigt(ii, jj), c)];
                    acc = cadd(acc, cscale(x[c], (c < 3 ? TE(1) : TE(2)) * s));
                }
                t[ii] = acc;
            }
        } else {
            // symmetric h (xx, yy, zz, yz, xz, xy): t_i = k_x h_xi + k_y h_yi + k_z h_zi
            t[0] = cadd(cadd(cscale(x[0], kv[0]), cscale(x[5], kv[1])), cscale(x[4], kv[2]));
            t[1] = cadd(cadd(cscale(x[5], kv[0]), cscale(x[1], kv[1])), cscale(x[3], kv[2]));
            t[2] = cadd(cadd(cscale(x[4], kv[0]), cscale(x[3], kv[1])), cscale(x[2], kv[2]));
        }
        T2 u[3];
        if (l >= kcnt || A.kt.cut(q, j, k) || (q == 0 && j == 0 && k == 0)) {
            u[0] = u[1] = u[2] = mk2<T2>(TE(0), TE(0));
        } else {
            green_u<TE>(A.ec.S, kv[0], kv[1], kv[2], t, u);
        }
        T2 v[3] = {u[0], u[1], u[2]};
        if (l < kcnt) {
            const long long o = base + q * es + l;
            const TE w = (k == 0 || ((A.g.Nz % 2) == 0 && k == A.g.Nz / 2)) ? TE(1) : TE(2);
            if (pre) green_update_in<TE>(A, o, gin, u, w, rd, rr, v);
            else green_update<TE>(A, o, u, w, rd, rr, v);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) oth[q * SP + c * TK + l] = strain_comp<TE>(c, kv[0], kv[1], kv[2], v);
    }
    if (A.resid) {
        AccSum2 s{double(rd), double(rr)};
        block_reduce_acc(s);
        if (threadIdx.x == 0)
            reinterpret_cast<AccSum2 *>(A.partials)[blockIdx.y * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
    T2 *r = fft_lines<TE, +1>(oth, cur, plan, tw, 6 * TK, SP, 1, false);
#pragma unroll
    for (int cmp = 0; cmp < 6; ++cmp) {
        for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
            const int q = e >> lgTK, l = e & (TK - 1);
            if (l < kcnt) A.E[cmp][base + q * es + l] = r[q * SP + cmp * TK + l];
        }
    }
}

// residual finalize: rel = sqrt(diff / max(ref, floor))
__global__ void k_resid_final(double *dscal, double floor_) {
    const double d = dscal[DS_RES_DIFF], r = dscal[DS_RES_REF];
    dscal[3] = sqrt(d / fmax(r, floor_));
}

// the stopping rule of the accelerated elastic solver on the device (loop
// control of main_cuda.cu:28982-29050): after an update, rel = sqrt(diff /
// max(ref, floor)); stop when iter >= iter_min and rel <= tol, at iter_max,
// or on a non-finite / negative residual sum.  Slots DS_EL + 0..3: done,
// updates taken, non-finite, converged.  Nothing changes once done is set.
__global__ void k_resid_step(double *dscal, double floor_, double tol, int iter_min, int iter_max) {
    double *st = dscal + DS_EL;
    if (st[0] != 0.0) return;
    const double d = dscal[DS_RES_DIFF], r = dscal[DS_RES_REF];
    const double it = st[1] + 1.0;
    st[1] = it;
    if (!isfinite(d) || !isfinite(r) || d < 0.0 || r < 0.0) {
        st[2] = 1.0;
        st[0] = 1.0;
        return;
    }
    const double rel = sqrt(d / fmax(r, floor_));
    dscal[3] = rel;
    if (it >= (double)iter_min && rel <= tol) {
        st[3] = 1.0;
        st[0] = 1.0;
    } else if (it >= (double)iter_max) {
        st[0] = 1.0;
    }
}

__global__ void k_el_status_reset(double *dscal) {
    if (threadIdx.x < 4) dscal[DS_EL + threadIdx.x] = 0.0;
}

// spectra a Green pass moves besides its 6 sources, 6 strains and 3 written
// displacements: the increment update reads r0, delta and u0 (and the
// Chebyshev iterate before delta); the first update writes r0 and delta
// (and zeroes that iterate); the plain form reads the old u for the residual
static int green_extra(const pfgb_ctx *c, int mode, int resid) {
    const bool cheb = c->Dkm[0] != nullptr;
    if (mode == 2) return cheb ? 12 : 9;
    if (mode == 1) return cheb ? 9 : 6;
    return resid ? 3 : 0;
}

template <typename TE>
static pfgb_status launch_green(pfgb_ctx *c, bool eigen, int resid, int *nblocks, int mode = 0) {
    using T2 = cplx_t<TE>;
    const int n = c->plx.n;
    auto bytes = [&](int tk) { return ((size_t)n + 2 * (size_t)n * (6 * tk + 1)) * sizeof(T2); };
    int TK = 16;
    while (TK > 1 && bytes(TK) > kSmemBudget) TK >>= 1;
    if (TK < 4 && sizeof(TE) == 4 && bytes(4) <= kSmemWide) TK = 4;
    while (TK > 1 && TK / 2 >= c->g.NzC) TK >>= 1;
    const size_t smem = bytes(TK);
    GreenArgs<TE> A;
    A.g = c->g;
    A.kt = KTab{c->kx, c->ky, c->kz, c->mx, c->my, c->mz};
    for (int i = 0; i < 21; ++i) { A.ec.S[i] = (TE)c->p.S[i]; A.ec.Sp[i] = (TE)c->p.S_p[i]; }
    A.tw = (const T2 *)c->tw[sizeof(TE) == 8 ? 0 : 1][0];
    for (int i = 0; i < 6; ++i) A.E[i] = (T2 *)c->E[i];
    for (int i = 0; i < 3; ++i) {
        A.U[i] = (T2 *)c->U[i]; A.R[i] = (T2 *)c->Rk[i]; A.D[i] = (T2 *)c->Dk[i]; A.Dm[i] = (T2 *)c->Dkm[i];
    }
    A.gam = (TE)c->cheb_gam;
    A.rho = (TE)c->cheb_rho;
    A.partials = c->partials;
    A.skip = c->skip;
    A.btab = (const float4 *)c->tc_btab;
    A.tc_err = c->tc_err;
    A.resid = resid;
    A.mode = mode;
    dim3 grid((c->g.NzC + TK - 1) / TK, c->g.Ny);
    // reads 6 source spectra (+3 old u for the residual), writes 3 u + 6 strain spectra
    ProfScope ps(c, {eigen ? "x_green_eigen" : "x_green_hij",
                     (double)(6 + 3 + 6 + green_extra(c, mode, resid)) * (double)c->g.Nk * sizeof(T2)});
    if (eigen) {
        auto kern = k_x_green<TE, true>;
        PFGB_CUDA_TRY(allow_smem(kern, smem));
        kern<<<grid, 256, smem, c->stream>>>(A, c->plx, TK);
    } else {
        auto kern = k_x_green<TE, false>;
        PFGB_CUDA_TRY(allow_smem(kern, smem));
        kern<<<grid, 256, smem, c->stream>>>(A, c->plx, TK);
    }
    PFGB_CUDA_TRY(cudaGetLastError());
    *nblocks = grid.x * grid.y;
    return PFGB_OK;
}

// ---------------------------------------------------------------------------
// elastic-iteration passes on 246-long axes (FP32, fft246.cuh engine): the
// same operations as k_x_green / k_zpass<OpHijZ> / the y OpCopy pass, with
// f246::NL lines per block in one in-place shared buffer
// ---------------------------------------------------------------------------
// TCS: the 41-point stages on the tensor cores (dft41_tc.cuh): shared memory
// B table | twiddles | line buffer without row padding
template <bool EIGEN, bool TCS>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_x_green246(GreenArgs<float> A) {
    if (A.skip && *A.skip != 0.0) return;
    using namespace f246;
    using T2 = float2;
    constexpr int TP = TC / 2;
    constexpr int PSX = TCS ? NL : PSTR;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t tc_mbar;
    __shared__ uint32_t tc_tbase;
    float4 *bt = reinterpret_cast<float4 *>(smem_raw);
    float2 *tw = reinterpret_cast<float2 *>(smem_raw + (TCS ? 2 * tc41::B_BYTES : 0));
    float2 *buf = tw + N;
    if constexpr (TCS) tc41::begin(&tc_tbase, &tc_mbar, bt, A.btab);
    const int k0 = blockIdx.x * TC, j = blockIdx.y;
    const int kcnt = min(TC, A.g.NzC - k0);
    const long long base = (long long)j * A.g.NzC + k0;
    const long long es = (long long)A.g.Ny * A.g.NzC;   // stride of x
    for (int e = threadIdx.x; e < 6 * N * TP; e += blockDim.x) {
        const int tp = e % TP, r = e / TP;
        const int q = r % N, s = r / N;
        const int t = 2 * tp;
        float2 *dst = buf + q * PSX + s * TC + t;
        const float2 *src = A.E[s] + base + q * es + t;
        if (t + 1 < kcnt) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src));
        } else {
            dst[0] = t < kcnt ? src[0] : make_float2(0.f, 0.f);
            dst[1] = make_float2(0.f, 0.f);
        }
    }
    cp_async_commit();
    load_twiddles(tw, A.tw);
    cp_async_wait_all();
    tc41::Ctx tcx{};
    if constexpr (TCS) {
        tcx = tc41::ready(&tc_tbase, &tc_mbar, bt, A.tc_err);
        tc41::lines<-1, PSX, 1>(buf, tw, tcx);
    } else {
        __syncthreads();
        lines<-1, PSX, 1>(buf, tw);
    }
    float rd = 0.f, rr = 0.f;
    // mode 2 (every iteration after the first of a step): the k-point's
    // r0 / delta / u0 / previous iterate are loaded as one batch first
    const bool pre = A.mode == 2;
    for (int e = threadIdx.x; e < N * TC; e += blockDim.x) {
        const int q = e / TC, l = e % TC, k = k0 + l;
        GreenIn<float> cur;
        if (pre && l < kcnt) green_fetch<float>(A, base + q * es + l, cur);
        const int kk = min(k, A.g.NzC - 1);
        const float kv[3] = {float(A.kt.kx[q]), float(A.kt.ky[j]), float(A.kt.kz[kk])};
        float2 *pt = buf + q * PSX + l;
        T2 x[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) x[c] = pt[c * TC];
        T2 t[3];
        if (EIGEN) {
#pragma unroll
            for (int ii = 0; ii < 3; ++ii) {
                T2 acc = make_float2(0.f, 0.f);
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    float sv = 0.f;
#pragma unroll
                    for (int jj = 0; jj < 3; ++jj) sv += kv[jj] * A.ec.S[vidx(tvoigt(ii, jj), c)];
                    acc = cadd(acc, cscale(x[c], (c < 3 ? 1.f : 2.f) * sv));
                }
                t[ii] = acc;
            }
        } else {
            t[0] = cadd(cadd(cscale(x[0], kv[0]), cscale(x[5], kv[1])), cscale(x[4], kv[2]));
            t[1] = cadd(cadd(cscale(x[5], kv[0]), cscale(x[1], kv[1])), cscale(x[3], kv[2]));
            t[2] = cadd(cadd(cscale(x[4], kv[0]), cscale(x[3], kv[1])), cscale(x[2], kv[2]));
        }
        T2 u[3];
        if (l >= kcnt || A.kt.cut(q, j, k) || (q == 0 && j == 0 && k == 0)) {
            u[0] = u[1] = u[2] = make_float2(0.f, 0.f);
        } else {
            green_u<float>(A.ec.S, kv[0], kv[1], kv[2], t, u);
        }
        T2 v[3] = {u[0], u[1], u[2]};
        if (l < kcnt) {
            const long long o = base + q * es + l;
            const float w = (k == 0 || ((A.g.Nz % 2) == 0 && k == A.g.Nz / 2)) ? 1.f : 2.f;
            if (pre) green_update_in<float>(A, o, cur, u, w, rd, rr, v);
            else green_update<float>(A, o, u, w, rd, rr, v);
        }
#pragma unroll
        for (int c = 0; c < 6; ++c) pt[c * TC] = strain_comp<float>(c, kv[0], kv[1], kv[2], v);
    }
    if (A.resid) {
        AccSum2 sacc{double(rd), double(rr)};
        block_reduce_acc(sacc);
        if (threadIdx.x == 0)
            reinterpret_cast<AccSum2 *>(A.partials)[blockIdx.y * gridDim.x + blockIdx.x] = sacc;
    }
    __syncthreads();
    if constexpr (TCS) tc41::lines<+1, PSX, 1>(buf, tw, tcx);
    else lines<+1, PSX, 1>(buf, tw);
    for (int e = threadIdx.x; e < 6 * N * TP; e += blockDim.x) {
        const int tp = e % TP, r = e / TP;
        const int q = r % N, s = r / N;
        const int t = 2 * tp;
        const float2 *srcs = buf + q * PSX + s * TC + t;
        float2 *dst = A.E[s] + base + q * es + t;
        if (t + 1 < kcnt) *reinterpret_cast<float4 *>(dst) = *reinterpret_cast<const float4 *>(srcs);
        else if (t < kcnt) dst[0] = srcs[0];
    }
    if constexpr (TCS) tc41::end(tcx.tmem);
}

// z pass with six fields in and six out (C2R -> op.point -> R2C), ZR rows
// per block: the rows' three field pairs are the block's NL complex lines
// TCS: the 41-point stages on the tensor cores (dft41_tc.cuh); shared
// memory B table | twiddles | lines
template <class Op, bool TCS>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_zpass246(Grid3 g, const float2 *tw_g, Op op, const double *skip, const float4 *btab, int *tc_err) {
    if (skip && *skip != 0.0) return;
    using namespace f246;
    constexpr int R = ZR, NC = N / 2 + 1;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t tc_mbar;
    __shared__ uint32_t tc_tbase;
    float4 *bt = reinterpret_cast<float4 *>(smem_raw);
    float2 *tw = reinterpret_cast<float2 *>(smem_raw + (TCS ? 2 * tc41::B_BYTES : 0));
    float2 *buf = tw + N;
    const long long row0 = (long long)blockIdx.x * R;
    const long long nrows = (long long)g.Nx * g.Ny;
    const int rcnt = (int)min((long long)R, nrows - row0);
    if constexpr (TCS) {
        tc41::begin(&tc_tbase, &tc_mbar, bt, btab);
        cp_async_commit();
    }
    load_twiddles(tw, tw_g);
    // unrolled by two: two trips' spectral loads in flight together
#pragma unroll 2
    for (int e = threadIdx.x; e < R * NC; e += blockDim.x) {
        const int rr = e / NC, k = e - rr * NC;
        float2 v[6];
        if (rr < rcnt) op.load_spec(row0 + rr, k, v);
        else {
#pragma unroll
            for (int f = 0; f < 6; ++f) v[f] = make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            float2 Av = v[2 * f], Bv = v[2 * f + 1];
            if (k == 0 || 2 * k == N) { Av.y = 0.f; Bv.y = 0.f; }
            float2 *line = buf + (rr * 3 + f) * N;
            // Z_k = A_k + i B_k ; Z_(n-k) = conj(A_k) + i conj(B_k)
            line[k] = make_float2(Av.x - Bv.y, Av.y + Bv.x);
            if (k > 0 && 2 * k != N) line[N - k] = make_float2(Av.x + Bv.y, Bv.x - Av.y);
        }
    }
    tc41::Ctx tcx{};
    if constexpr (TCS) {
        cp_async_wait_all();
        tcx = tc41::ready(&tc_tbase, &tc_mbar, bt, tc_err);
        tc41::lines<+1, 1, N>(buf, tw, tcx);
    } else {
        __syncthreads();
        lines<+1, 1, N>(buf, tw);
    }
    typename Op::Acc acc = Op::Acc::identity();
    for (int e = threadIdx.x; e < rcnt * N; e += blockDim.x) {
        const int r = e / N, z = e - r * N;
        float vi[6], vo[6];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float2 w = buf[(r * 3 + f) * N + z];
            vi[2 * f] = w.x;
            vi[2 * f + 1] = w.y;
        }
        op.point((row0 + r) * N + z, vi, vo, acc);
#pragma unroll
        for (int f = 0; f < 3; ++f) buf[(r * 3 + f) * N + z] = make_float2(vo[2 * f], vo[2 * f + 1]);
    }
    if constexpr (Op::Acc::kActive) {
        block_reduce_acc(acc);
        if (threadIdx.x == 0) op.finish(blockIdx.x, acc);
    }
    __syncthreads();
    if constexpr (TCS) tc41::lines<-1, 1, N>(buf, tw, tcx);
    else lines<-1, 1, N>(buf, tw);
    for (int e = threadIdx.x; e < rcnt * NC; e += blockDim.x) {
        const int rr = e / NC, k = e - rr * NC;
        float2 v[6];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const float2 *line = buf + (rr * 3 + f) * N;
            const float2 Zk = line[k], Zm = line[k == 0 ? 0 : N - k];
            // A_k = (Z_k + conj Z_-k) / 2 ; B_k = (Z_k - conj Z_-k) / (2 i)
            v[2 * f] = make_float2(0.5f * (Zk.x + Zm.x), 0.5f * (Zk.y - Zm.y));
            v[2 * f + 1] = make_float2(0.5f * (Zk.y + Zm.y), 0.5f * (Zm.x - Zk.x));
        }
        op.store_spec(row0 + rr, k, v);
    }
    if constexpr (TCS) tc41::end(tcx.tmem);
}

template <int DIR>
static pfgb_status launch_y246(pfgb_ctx *c, const char *tag) {
    if (c->tc_y) {   // the 41-point stage on the tensor cores
        const size_t smem = tc41::y_smem_bytes();
        auto kern = k_y246tc<DIR>;
        PFGB_CUDA_TRY(allow_smem(kern, smem));
        AxisIO<float, 6, 6> io;
        for (int i = 0; i < 6; ++i) { io.in[i] = (const float2 *)c->E[i]; io.out[i] = (float2 *)c->E[i]; }
        dim3 grid((c->g.NzC + f246::TC - 1) / f246::TC, c->g.Nx);
        ProfScope ps(c, {tag, 12.0 * (double)c->g.Nk * sizeof(float2)});
        kern<<<grid, f246::THREADS, smem, c->stream>>>(c->g, (const float2 *)c->tw[1][1], (const float4 *)c->tc_btab,
                                                       io, c->skip, c->tc_err);
        PFGB_CUDA_TRY(cudaGetLastError());
        return PFGB_OK;
    }
    const size_t smem = f246::axis_smem_bytes();
    auto kern = k_y246<DIR>;
    PFGB_CUDA_TRY(allow_smem(kern, smem));
    AxisIO<float, 6, 6> io;
    for (int i = 0; i < 6; ++i) { io.in[i] = (const float2 *)c->E[i]; io.out[i] = (float2 *)c->E[i]; }
    dim3 grid((c->g.NzC + f246::YC - 1) / f246::YC, c->g.Nx, 6 / f246::YS);
    ProfScope ps(c, {tag, 12.0 * (double)c->g.Nk * sizeof(float2)});
    kern<<<grid, f246::THREADS, smem, c->stream>>>(c->g, (const float2 *)c->tw[1][1], io, c->skip);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

static pfgb_status launch_green246(pfgb_ctx *c, bool eigen, int resid, int *nblocks, int mode = 0) {
    const size_t smem = f246::axis_smem_bytes();
    GreenArgs<float> A;
    A.g = c->g;
    A.kt = KTab{c->kx, c->ky, c->kz, c->mx, c->my, c->mz};
    for (int i = 0; i < 21; ++i) { A.ec.S[i] = (float)c->p.S[i]; A.ec.Sp[i] = (float)c->p.S_p[i]; }
    A.tw = (const float2 *)c->tw[1][0];
    for (int i = 0; i < 6; ++i) A.E[i] = (float2 *)c->E[i];
    for (int i = 0; i < 3; ++i) {
        A.U[i] = (float2 *)c->U[i]; A.R[i] = (float2 *)c->Rk[i]; A.D[i] = (float2 *)c->Dk[i];
        A.Dm[i] = (float2 *)c->Dkm[i];
    }
    A.gam = (float)c->cheb_gam;
    A.rho = (float)c->cheb_rho;
    A.partials = c->partials;
    A.skip = c->skip;
    A.btab = (const float4 *)c->tc_btab;
    A.tc_err = c->tc_err;
    A.resid = resid;
    A.mode = mode;
    dim3 grid((c->g.NzC + f246::TC - 1) / f246::TC, c->g.Ny);
    ProfScope ps(c, {eigen ? "x_green_eigen" : "x_green_hij",
                     (double)(6 + 3 + 6 + green_extra(c, mode, resid)) * (double)c->g.Nk * sizeof(float2)});
    auto go = [&](auto kern, size_t sm) -> pfgb_status {
        PFGB_CUDA_TRY(allow_smem(kern, sm));
        kern<<<grid, f246::THREADS, sm, c->stream>>>(A);
        return PFGB_OK;
    };
    if (c->tc_x) {   // the 41-point stages on the tensor cores
        const size_t smem_tc = tc41::y_smem_bytes();
        TRY(eigen ? go(k_x_green246<true, true>, smem_tc) : go(k_x_green246<false, true>, smem_tc));
    } else {
        TRY(eigen ? go(k_x_green246<true, false>, smem) : go(k_x_green246<false, false>, smem));
    }
    PFGB_CUDA_TRY(cudaGetLastError());
    *nblocks = grid.x * grid.y;
    return PFGB_OK;
}

template <class Op>
static pfgb_status launch_z246(pfgb_ctx *c, Op op, const char *tag, double extra_bytes) {
    const size_t smem = f246::z_smem_bytes();
    const long long rows = (long long)c->g.Nx * c->g.Ny;
    const int nb = (int)((rows + f246::ZR - 1) / f246::ZR);
    ProfScope ps(c, {tag, 12.0 * (double)c->g.Nk * sizeof(float2) + extra_bytes});
    if (c->tc_z) {   // the 41-point stages on the tensor cores
        auto kern = k_zpass246<Op, true>;
        const size_t smem_tc = 2 * tc41::B_BYTES + smem;
        PFGB_CUDA_TRY(allow_smem(kern, smem_tc));
        kern<<<nb, f246::THREADS, smem_tc, c->stream>>>(c->g, (const float2 *)c->tw[1][2], op, c->skip,
                                                         (const float4 *)c->tc_btab, c->tc_err);
    } else {
        auto kern = k_zpass246<Op, false>;
        PFGB_CUDA_TRY(allow_smem(kern, smem));
        kern<<<nb, f246::THREADS, smem, c->stream>>>(c->g, (const float2 *)c->tw[1][2], op, c->skip, nullptr,
                                                     nullptr);
    }
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// ===========================================================================
// step orchestration
// ===========================================================================
template <typename T, typename TE>
static DevState<T, TE> dev_state(pfgb_ctx *c) {
    DevState<T, TE> d;
    d.g = c->g;
    d.kt = KTab{c->kx, c->ky, c->kz, c->mx, c->my, c->mz};
    d.phi_old = (T *)c->phi[c->cur];
    d.phi_new = (T *)c->phi[1 - c->cur];
    d.eta_old = (T *)c->eta[c->ecur];
    d.eta_new = (T *)c->eta[1 - c->ecur];
    d.Y = (T *)c->Y;
    d.Yprev = (T *)c->Yprev;
    d.q = (T *)c->q;
    d.qb = (T *)c->qb;
    d.divr = (T *)c->divr;
    for (int i = 0; i < 6; ++i) d.sig[i] = (TE *)c->sig[i];
    d.mge = (T *)c->mge;
    d.mlap = (T *)c->mlap;
    d.dYdt = (T *)c->dYdt;
    for (int i = 0; i < 6; ++i) { d.eps[i] = (TE *)c->eps[i]; d.E[i] = (cplx_t<TE> *)c->E[i]; }
    for (int i = 0; i < 3; ++i) d.U[i] = (cplx_t<TE> *)c->U[i];
    for (int i = 0; i < 4; ++i) d.S[i] = (cplx_t<T> *)c->S[i];
    d.partials = c->partials;
    d.dscal = c->dscal;
    d.Yc = c->Yc;
    d.dYoff = c->dYoff;
    return d;
}

template <typename TE>
static ElasC<TE> elas_consts(const pfgb_ctx *c) {
    ElasC<TE> e;
    for (int i = 0; i < 21; ++i) { e.S[i] = (TE)c->p.S[i]; e.Sp[i] = (TE)c->p.S_p[i]; }
    for (int i = 0; i < 6; ++i) { e.e00[i] = (TE)c->p.eps00[i]; e.E0[i] = (TE)c->p.E0[i]; }
    e.invN = (TE)(1.0 / (double)c->g.N);
    return e;
}

static pfgb_status sync_read(pfgb_ctx *c, int first, int count) {
    PFGB_CUDA_TRY(cudaMemcpyAsync(c->hscal + first, c->dscal + first, sizeof(double) * count,
                                  cudaMemcpyDeviceToHost, c->stream));
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PFGB_OK;
}

template <typename TE>
__global__ void k_add_increment(cplx_t<TE> *u0, cplx_t<TE> *u1, cplx_t<TE> *u2, const cplx_t<TE> *d0,
                                const cplx_t<TE> *d1, const cplx_t<TE> *d2, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        u0[i] = cadd(u0[i], d0[i]);
        u1[i] = cadd(u1[i], d1[i]);
        u2[i] = cadd(u2[i], d2[i]);
    }
}

// the warm start from the last solutions: the polynomial extrapolation of
// order m through u^n and the history h[0..m-1] = u^{n-1}, ..., u^{n-m}
// (1: 2 u^n - u^{n-1}; 2: 3 u^n - 3 u^{n-1} + u^{n-2}; 3: 4, -6, 4, -1;
// 4: 5, -10, 10, -5, 1; 5: 6, -15, 20, -15, 6, -1), formed as u^n plus its
// backward differences
// (nabla u^n + nabla^2 u^n + ... + nabla^m u^n): the differences of
// neighbouring solutions are small and nearly exact in the field type, so
// the sum loses less than the binomial form would.  u^n is also written to
// `slot`, the history level that becomes u^{n-1} (the host rotates the
// levels' pointers instead of copying them).
template <typename TE>
struct ExtrapArgs { cplx_t<TE> *u[3], *h[5][3], *slot[3]; };
template <typename TE>
__global__ void k_extrapolate_u(ExtrapArgs<TE> a, long long n, int m) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            cplx_t<TE> d[6];
            d[0] = a.u[c][i];
#pragma unroll
            for (int l = 0; l < 5; ++l)
                if (l < m) d[l + 1] = a.h[l][c][i];
            a.slot[c][i] = d[0];
            if (m >= 1) {
                // d[j] <- nabla^j u^n, level by level
                cplx_t<TE> sum = d[0];
#pragma unroll
                for (int k = 1; k <= 5; ++k) {
                    if (k > m) break;
#pragma unroll
                    for (int l = 5; l >= 1; --l)
                        if (l >= k && l <= m) d[l] = mk2<cplx_t<TE>>(d[l - 1].x - d[l].x, d[l - 1].y - d[l].y);
                    sum = mk2<cplx_t<TE>>(sum.x + d[k].x, sum.y + d[k].y);
                }
                a.u[c][i] = sum;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// learned start of the heterogeneous iteration (no reference counterpart;
// the reference's warm-start point is main_cuda.cu:28792-28870)
// ---------------------------------------------------------------------------
// model inputs: phi, eta and the 6 eigenstrain components the cold start's
// eigenstrain pass sees (OpEigenR2C), as float [8][N]
template <typename T, typename TE>
__global__ void k_fno_inputs(DevState<T, TE> d, PhysCT<T> c, ElasC<TE> ec, float *__restrict__ out) {
    const long long N = d.g.N;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < N;
         n += (long long)gridDim.x * blockDim.x) {
        const T xB = xB_of_Y<T>(c, d.Y[n] + T(d.Yc));
        const T phi = d.phi_old[n], eta = c.gp ? d.eta_old[n] : T(0);
        TE e0[6];
        eigenstrain<T, TE>(c, ec, phi, eta, xB_el(c, xB), c.gp_el != 0, e0);
        out[n] = (float)phi;
        out[N + n] = (float)eta;
#pragma unroll
        for (int a = 0; a < 6; ++a) out[(2 + a) * N + n] = (float)e0[a];
    }
}

// z r2c of three real float fields into E[0..2]
template <typename TE>
struct OpReal3In {
    using Acc = NoAcc;
    const float *src; cplx_t<TE> *E0, *E1, *E2; long long N; int NzC;
    __device__ void point(long long cell, const TE *, TE *out, Acc &) const {
        out[0] = (TE)src[cell];
        out[1] = (TE)src[N + cell];
        out[2] = (TE)src[2 * N + cell];
    }
    __device__ void load_spec(long long, int, cplx_t<TE> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<TE> *v) const {
        const long long o = row * NzC + k;
        E0[o] = v[0]; E1[o] = v[1]; E2[o] = v[2];
    }
};
// z c2r of E[0..2] into three real float fields, times 1/N
template <typename TE>
struct OpReal3Out {
    using Acc = NoAcc;
    const cplx_t<TE> *E0, *E1, *E2; float *dst; long long N; int NzC; TE invN;
    __device__ void load_spec(long long row, int k, cplx_t<TE> *v) const {
        const long long o = row * NzC + k;
        v[0] = E0[o]; v[1] = E1[o]; v[2] = E2[o];
    }
    __device__ void point(long long cell, const TE *in, TE *, Acc &) const {
        dst[cell] = (float)(in[0] * invN);
        dst[N + cell] = (float)(in[1] * invN);
        dst[2 * N + cell] = (float)(in[2] * invN);
    }
    __device__ void store_spec(long long, int, const cplx_t<TE> *) const {}
};
// x pass of the displacement correction: dealiased like u, u(k = 0) = 0
template <typename TE>
struct OpCutU3 {
    static constexpr bool kInplace = false;
    KTab kt;
    __device__ void apply(int i, int j, int k, const cplx_t<TE> *in, cplx_t<TE> *out) const {
        const bool z = kt.cut(i, j, k) || (i == 0 && j == 0 && k == 0);
#pragma unroll
        for (int a = 0; a < 3; ++a) out[a] = z ? mk2<cplx_t<TE>>(TE(0), TE(0)) : in[a];
    }
};
template <typename TE>
__global__ void k_sub3(cplx_t<TE> *d0, cplx_t<TE> *d1, cplx_t<TE> *d2, const cplx_t<TE> *u0, const cplx_t<TE> *u1,
                       const cplx_t<TE> *u2, const cplx_t<TE> *h0, const cplx_t<TE> *h1, const cplx_t<TE> *h2,
                       long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        d0[i] = csub(u0[i], h0[i]);
        d1[i] = csub(u1[i], h1[i]);
        d2[i] = csub(u2[i], h2[i]);
    }
}

template <typename T, typename TE>
static pfgb_status launch_fno_inputs(pfgb_ctx *c, float *out) {
    ProfScope ps(c, {"model_inputs", (double)c->g.N * (3.0 * sizeof(T) + 8.0 * sizeof(float))});
    k_fno_inputs<T, TE><<<1216, 256, 0, c->stream>>>(dev_state<T, TE>(c), phys_as<T>(c->pc), elas_consts<TE>(c), out);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// U <- U + FFT(model prediction), E[0..2] as scratch
template <typename T, typename TE>
static pfgb_status model_start(pfgb_ctx *c) {
    using T2e = cplx_t<TE>;
    const double Nf = (double)c->g.N;
    TRY((launch_fno_inputs<T, TE>(c, c->fno_in)));
    TRY(pfgb_fno_set_stream(c->fno, c->stream));
    {
        ProfScope ps(c, {"model_forward", 0.0});
        c->launches += pfgb_fno_forward_launches(c->fno) - 1;
        TRY(pfgb_fno_forward(c->fno, c->fno_in, c->fno_out));
    }
    T2e *E0 = (T2e *)c->E[0], *E1 = (T2e *)c->E[1], *E2 = (T2e *)c->E[2];
    TRY((launch_z<TE, 0, 3>(c, OpReal3In<TE>{c->fno_out, E0, E1, E2, c->g.N, c->g.NzC}, "z_model_r2c",
                            3.0 * Nf * sizeof(float))));
    AxisIO<TE, 3, 3> io;
    for (int i = 0; i < 3; ++i) { io.in[i] = (const T2e *)c->E[i]; io.out[i] = (T2e *)c->E[i]; }
    TRY((launch_axis<TE, 3, 3, -1, 0>(c, 1, io, OpCopy<TE, 3>{}, "y_fwd3")));
    TRY((launch_axis<TE, 3, 3, -1, 0>(c, 2, io, OpCutU3<TE>{KTab{c->kx, c->ky, c->kz, c->mx, c->my, c->mz}},
                                      "x_fwd3")));
    ProfScope ps(c, {"add_increment", 9.0 * (double)c->g.Nk * sizeof(T2e)});
    k_add_increment<TE><<<1216, 256, 0, c->stream>>>((T2e *)c->U[0], (T2e *)c->U[1], (T2e *)c->U[2], E0, E1, E2,
                                                     c->g.Nk);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

template <typename T, typename TE>
static pfgb_status elastic_solve(pfgb_ctx *c, pfgb_step_stats *st) {
    using T2e = cplx_t<TE>;
    const pfgb_params &P = c->p;
    const PhysCT<T> pc = phys_as<T>(c->pc);
    const ElasC<TE> ec = elas_consts<TE>(c);
    DevState<T, TE> d = dev_state<T, TE>(c);
    const KTab kt = d.kt;
    const int accel = P.elastic_enabled && (P.elastic_warm_start_enabled || P.elastic_residual_control_enabled);
    const int src = P.elastic_warm_start_source;
    const int use_model = accel && !c->pair_mode && c->fno && (src == 2 || (src == 1 && !c->warm_valid));
    const int warm_used = accel && !c->pair_mode && !use_model && c->warm_valid && src <= 1;
    const double Nf = (double)c->g.N;
    AxisIO<TE, 6, 6> io6;
    for (int i = 0; i < 6; ++i) { io6.in[i] = (const T2e *)c->E[i]; io6.out[i] = (T2e *)c->E[i]; }
    int nb = 0;
    // the four passes of an iteration, on the 246-point engine where the axis allows
    auto ypass = [&](int dir, const char *tag) -> pfgb_status {
        if constexpr (std::is_same<TE, float>::value) {
            if (c->f246[1]) return dir < 0 ? launch_y246<-1>(c, tag) : launch_y246<+1>(c, tag);
        }
        return dir < 0 ? launch_axis<TE, 6, 6, -1, 0>(c, 1, io6, OpCopy<TE, 6>{}, tag)
                       : launch_axis<TE, 6, 6, +1, 0>(c, 1, io6, OpCopy<TE, 6>{}, tag);
    };
    auto green = [&](bool eigen, int resid, int mode) -> pfgb_status {
        if constexpr (std::is_same<TE, float>::value) {
            if (c->f246[0]) return launch_green246(c, eigen, resid, &nb, mode);
        }
        return launch_green<TE>(c, eigen, resid, &nb, mode);
    };
    auto hij = [&](int lin) -> pfgb_status {
        const double extra = lin ? 2.0 * Nf * sizeof(T) : (2.0 + pc.gp) * Nf * sizeof(T);
        if constexpr (std::is_same<TE, float>::value) {
            if (c->f246[2]) return launch_z246(c, OpHijZ<T, TE>{d, pc, ec, lin}, "z_hij", extra);
        }
        return launch_z<TE, 6, 6>(c, OpHijZ<T, TE>{d, pc, ec, lin}, "z_hij", extra);
    };
    // increment form: one full update, then delta <- r0 + L delta
    const int inc = accel && P.elastic_increment_form && c->Rk[0] != nullptr;
    if (accel && (src == 1 || src == 2) && !c->pair_mode && !c->fno && (src == 2 || !c->warm_valid)) {
        pfgb_set_error_msg("elastic_warm_start_source=%d needs a model (pfgb_set_warm_start_model)", src);
        return PFGB_ERR_INVALID;
    }
    if (!warm_used) {
        TRY((launch_z<TE, 0, 6>(c, OpEigenR2C<T, TE>{d, pc, ec}, "z_eigen_r2c", (2.0 + pc.gp) * Nf * sizeof(T))));
        TRY(ypass(-1, "y_fwd6"));
        TRY(green(true, 0, 0));
        if (c->pair_mode)
            for (int i = 0; i < 3; ++i)
                PFGB_CUDA_TRY(cudaMemcpyAsync(c->Uhom[i], c->U[i], sizeof(T2e) * c->g.Nk, cudaMemcpyDeviceToDevice,
                                              c->stream));
    }
    if (use_model) TRY((model_start<T, TE>(c)));
    if (warm_used || use_model) {
        if (warm_used && c->Uhist[0][0]) {
            // u0 extrapolated through the last m + 1 solutions, m the order
            // or fewer while the history fills; u^n goes into the oldest
            // level, which the pointer rotation below makes u^{n-1}
            const int nh = P.elastic_warm_start_extrapolate;
            const int m = std::min(nh, c->warm_count - 1);
            ProfScope ps(c, {"extrapolate_u", (3.0 + (double)std::max(m, 0)) * 3.0 * (double)c->g.Nk * sizeof(T2e)});
            ExtrapArgs<TE> a;
            for (int i = 0; i < 3; ++i) {
                a.u[i] = (T2e *)c->U[i];
                for (int l = 0; l < 5; ++l) a.h[l][i] = (T2e *)c->Uhist[l][i];
                a.slot[i] = (T2e *)c->Uhist[nh - 1][i];
            }
            k_extrapolate_u<TE><<<1216, 256, 0, c->stream>>>(a, c->g.Nk, std::max(m, 0));
            PFGB_CUDA_TRY(cudaGetLastError());
            for (int i = 0; i < 3; ++i) {
                void *oldest = c->Uhist[nh - 1][i];
                for (int l = nh - 1; l > 0; --l) c->Uhist[l][i] = c->Uhist[l - 1][i];
                c->Uhist[0][i] = oldest;
            }
        }
        AxisIO<TE, 3, 6> io;
        for (int i = 0; i < 3; ++i) io.in[i] = (const T2e *)c->U[i];
        for (int i = 0; i < 6; ++i) io.out[i] = (T2e *)c->E[i];
        TRY((launch_axis<TE, 3, 6, 0, +1>(c, 2, io, OpStrainFromUX<TE>{kt}, "x_strain_from_u")));
    }
    TRY(ypass(+1, "y_inv6"));
    int iter = accel ? 0 : 1;
    int conv = accel ? 0 : 1;
    double rel = NAN;
    // Chebyshev semi-iteration of the increment (elastic_chebyshev): rho of
    // each update from the recurrence rho_2 = 2 / (2 - sig^2),
    // rho_{k+1} = 1 / (1 - sig^2 rho_k / 4); the new iterate is written over
    // the one before, so the two buffers swap after every update
    const bool cheb = inc && c->Dkm[0] != nullptr;
    int cheb_it = 0;
    // one update of the fixed point (iteration index k from 0)
    auto update = [&](int k) -> pfgb_status {
        const int lin = inc && k >= 1;
        TRY(hij(lin));
        TRY(ypass(-1, "y_fwd6"));
        if (cheb && lin) {
            const double s2 = c->cheb_sig * c->cheb_sig;
            c->cheb_rho = cheb_it == 0 ? 2.0 / (2.0 - s2) : 1.0 / (1.0 - 0.25 * s2 * c->cheb_rho);
            ++cheb_it;
        }
        TRY(green(false, accel, inc ? (lin ? 2 : 1) : 0));
        if (cheb && lin)
            for (int i = 0; i < 3; ++i) std::swap(c->Dk[i], c->Dkm[i]);
        return ypass(+1, "y_inv6");
    };
    if (accel) {
        // The residual test runs on the device (k_resid_step) and the host
        // launches the updates in batches, reading the status once per
        // batch: the first batch is the last solve's count (with the
        // extrapolated start the count moves by one at most from step to
        // step, so one read usually ends the solve), later ones two.
        // Updates launched past the stopping point return at once
        // (c->skip): an unneeded update costs its empty launches, a second
        // batch a host round trip.  The Chebyshev buffer swaps the host made
        // for updates that returned at once are undone below.
        struct SkipGuard { pfgb_ctx *c; ~SkipGuard() { c->skip = nullptr; } } guard{c};
        k_el_status_reset<<<1, 32, 0, c->stream>>>(c->dscal);
        PFGB_CUDA_TRY(cudaGetLastError());
        c->skip = c->dscal + DS_EL;
        const int imax = std::max(1, P.elastic_iter_max);
        int batch = c->last_el_iters > 1 ? c->last_el_iters : 4;
        batch = std::max(1, std::min(std::max(batch, P.elastic_iter_min), imax));
        int launched = 0;
        for (;;) {
            const int nbat = std::min(batch, imax - launched);
            for (int b = 0; b < nbat; ++b) {
                TRY(update(launched + b));
                TRY(reduce_to<AccSum2>(c, nb, DS_RES_DIFF));
                k_resid_step<<<1, 1, 0, c->stream>>>(c->dscal, P.elastic_residual_absolute_floor,
                                                     P.elastic_residual_tolerance, P.elastic_iter_min, imax);
                PFGB_CUDA_TRY(cudaGetLastError());
            }
            launched += nbat;
            PFGB_CUDA_TRY(cudaMemcpyAsync(c->hscal + 3, c->dscal + 3, sizeof(double), cudaMemcpyDeviceToHost,
                                          c->stream));
            TRY(sync_read(c, DS_EL, 4));
            if (c->hscal[DS_EL] != 0.0 || launched >= imax) break;
            batch = 2;
        }
        c->skip = nullptr;
        if (c->tc_err) {   // a bounded wait of the tensor-core stage ran out
            int te = 0;
            PFGB_CUDA_TRY(cudaMemcpy(&te, c->tc_err, sizeof(int), cudaMemcpyDeviceToHost));
            if (te) {
                pfgb_set_error_msg("tensor-core 41-point stage: a wait for the MMA completion ran out at step %d",
                                   c->step + 1);
                return PFGB_ERR_TIMEOUT;
            }
        }
        iter = (int)c->hscal[DS_EL + 1];
        conv = c->hscal[DS_EL + 3] != 0.0;
        rel = c->hscal[3];
        if (cheb) {
            // the host swapped after every launched linear update; the device
            // ran iter updates (linear from the second on)
            const int done_swaps = std::max(0, iter - 1), host_swaps = std::max(0, launched - 1);
            if ((host_swaps - done_swaps) % 2 != 0)
                for (int i = 0; i < 3; ++i) std::swap(c->Dk[i], c->Dkm[i]);
        }
        if (c->hscal[DS_EL + 2] != 0.0) {
            pfgb_set_error_msg("elastic residual is non-finite at step %d", c->step + 1);
            return PFGB_ERR_NONFINITE;
        }
        c->last_el_iters = iter;
    } else {
        for (;;) {
            TRY(update(iter));
            ++iter;
            if (iter >= P.elastic_iter_max) break;
        }
    }
    if (accel) { c->warm_valid = 1; c->warm_count++; }
    c->el_iterations = (uint64_t)iter;
    c->el_residual = rel;
    if (st) {
        st->elastic_iterations = iter;
        st->elastic_converged = conv;
        st->elastic_warm_start_used = use_model ? 2 : warm_used;
        st->elastic_relative_residual = rel;
        st->elastic_iterations_total += iter;
    }
    if (accel && !conv && P.elastic_fail_on_nonconvergence) {
        pfgb_set_error_msg("elastic solver did not converge at step %d: iterations=%d residual=%.17e",
                           c->step + 1, iter, rel);
        return PFGB_ERR_NONCONVERGED;
    }
    if (inc) {
        // u = u0 + delta, and the strain of u for the final pass
        {
            ProfScope ps(c, {"add_increment", 9.0 * (double)c->g.Nk * sizeof(T2e)});
            k_add_increment<TE><<<1216, 256, 0, c->stream>>>((T2e *)c->U[0], (T2e *)c->U[1], (T2e *)c->U[2],
                                                             (const T2e *)c->Dk[0], (const T2e *)c->Dk[1],
                                                             (const T2e *)c->Dk[2], c->g.Nk);
            PFGB_CUDA_TRY(cudaGetLastError());
        }
        AxisIO<TE, 3, 6> io;
        for (int i = 0; i < 3; ++i) io.in[i] = (const T2e *)c->U[i];
        for (int i = 0; i < 6; ++i) io.out[i] = (T2e *)c->E[i];
        TRY((launch_axis<TE, 3, 6, 0, +1>(c, 2, io, OpStrainFromUX<TE>{kt}, "x_strain_from_u")));
        TRY(ypass(+1, "y_inv6"));
    }
    TRY((launch_z<TE, 6, 0>(c, OpStrainFinalZ<T, TE>{d, ec, pc}, "z_strain_final",
                                (d.sig[0] ? 12.0 : 6.0) * Nf * sizeof(TE))));
    return PFGB_OK;
}

// zero-mode solve (run_pf_conserved_y_zero_mode_host, main_cuda.cu:4269-4405):
// the same bracket check and Newton / bisection iteration on
// F(l) = sum((1-h) sigmoid(Y* + l) + h v_B) - target.  The Newton iterates
// are first taken on the quartic Taylor model of F about l = 0 (moments
// accumulated by the final Y pass, no extra pass); the iteration is then
// continued on FP64 direct evaluations until |F| <= tol, so convergence is
// always decided on the exact sum, as in the reference.
template <typename T, typename TE>
static pfgb_status zero_mode(pfgb_ctx *c, int nb_final, pfgb_step_stats *st) {
    const pfgb_params &P = c->p;
    TRY(reduce_to<AccZM>(c, nb_final, DS_ZM));
    TRY(sync_read(c, DS_MEAN_DY, DS_ZM + 8));   // mean_DY rides along
    const double ymin = c->hscal[DS_ZM] + c->Yc, ymax = c->hscal[DS_ZM + 1] + c->Yc;
    double M[5];
    for (int i = 0; i < 5; ++i) M[i] = c->hscal[DS_ZM + 2 + i];
    c->sum_alpha = c->hscal[DS_ZM + 7] * (1.0 + 1e-4);   // FP32 partial sums: generous margin
    const double Ycap = P.Y_clip;
    auto fail = [&](const char *why) {
        pfgb_set_error_msg("PF zero-mode rejected step=%d: %s", c->step + 1, why);
        return PFGB_ERR_ZERO_MODE;
    };
    if (!std::isfinite(ymin) || !std::isfinite(ymax)) return fail("non-finite Y*");
    double lo = -P.Y_clip - ymin, hi = Ycap - ymax;
    const double rnd = 128.0 * 2.220446049250313e-16 * std::max(std::max(std::fabs(lo), std::fabs(hi)), 1.0);
    if (!std::isfinite(lo) || !std::isfinite(hi) || lo > hi + rnd) return fail("empty lambda interval");
    const double target = c->target_mass;
    const double tol = P.zero_mode_tolerance_relative * std::max(std::fabs(target), 1.0);
    const long long N = c->g.N;
    auto direct = [&](const double *lams, int nl, double *mass, double *der, bool exact = true) -> pfgb_status {
        if (nl < 1 || nl > 2) return fail("internal: 1 or 2 trial multipliers per evaluation");
        PFGB_CUDA_TRY(cudaMemcpyAsync(c->dscal + DS_EV, lams, sizeof(double) * nl, cudaMemcpyHostToDevice, c->stream));
        // FP32 fields: the exact evaluation in double-float unless
        // zero_mode_fp64_cells asks for FP64 per cell; that kernel is an
        // arithmetic chain per cell and takes 8 blocks per SM, the others 2
        const bool dfe = sizeof(T) == 4 && exact && !P.zero_mode_fp64_cells;
        const int eb = dfe ? 1216 : 304;
        {
            ProfScope ps(c, {"zero_mode_eval", (double)N * 2.0 * sizeof(T)});
            const T *Yp = (const T *)c->Y, *ph = (const T *)c->phi[1 - c->cur];
            const double *lp = c->dscal + DS_EV;
            if constexpr (sizeof(T) == 4) {
                if (dfe && nl == 2) k_zm_eval_df<2><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
                else if (dfe) k_zm_eval_df<1><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
            }
            if (dfe) {
            } else if (exact && nl == 2) k_zm_eval<T, double, 2><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
            else if (exact) k_zm_eval<T, double, 1><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
            else if (nl == 2) k_zm_eval<T, T, 2><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
            else k_zm_eval<T, T, 1><<<eb, 256, 0, c->stream>>>(Yp, ph, N, c->Yc, P.v_B, lp, c->partials);
        }
        PFGB_CUDA_TRY(cudaGetLastError());
        for (int q = 0; q < nl; ++q) {
            ProfScope ps(c, {"reduce_partials", (double)eb * sizeof(AccSum2)});
            k_reduce_partials<AccSum2><<<1, 256, 0, c->stream>>>((const AccSum2 *)c->partials + q * eb, eb,
                                                                 c->dscal, DS_BR + 2 * q, 1.0);
        }
        PFGB_CUDA_TRY(cudaGetLastError());
        TRY(sync_read(c, DS_BR, 2 * nl));
        for (int q = 0; q < nl; ++q) { mass[q] = c->hscal[DS_BR + 2 * q]; der[q] = c->hscal[DS_BR + 2 * q + 1]; }
        return PFGB_OK;
    };
    // the reference's bracket test: mass(lo) <= target + tol and
    // mass(hi) >= target - tol.  Evaluated only when the iteration does not
    // reach the tolerance, to name the failure: mass is increasing in the
    // shift, so an accepted point inside [lo, hi] (evaluated or certified
    // within tol) already implies both conditions.
    const double lo0 = lo, hi0 = hi;
    auto check_bracket = [&]() -> pfgb_status {
        // bracket ends: evaluated in field precision; an FP64 re-evaluation is
        // taken only when the FP32 value is within 1e-5 of the decision limit
        double ls[2] = {lo0, hi0}, ms[2], ds[2];
        const bool fp32 = sizeof(T) == 4;
        TRY(direct(ls, 2, ms, ds, !fp32));
        if (fp32) {
            const double margin = 1e-5 * std::max(std::fabs(target), 1.0);
            if (!std::isfinite(ms[0]) || !std::isfinite(ms[1]) || std::fabs(ms[0] - target - tol) < margin ||
                std::fabs(ms[1] - target + tol) < margin)
                TRY(direct(ls, 2, ms, ds, true));
        }
        if (!std::isfinite(ms[0]) || !std::isfinite(ms[1])) return fail("non-finite bracket mass");
        if (ms[0] - target > tol || ms[1] - target < -tol) return fail("target outside bracket");
        return PFGB_OK;
    };
    int iters = 0, nwt = 0, bis = 0;
    // one safeguarded Newton / bisection update (same rule as the reference)
    auto update = [&](double &lam, double res, double der) {
        if (res < 0.0) lo = lam; else hi = lam;
        double cand = NAN;
        if (der > 0.0 && std::isfinite(der)) cand = lam - res / der;
        if (std::isfinite(cand) && cand > lo && cand < hi) ++nwt;
        else { cand = 0.5 * (lo + hi); ++bis; }
        lam = cand;
    };
    double lam = std::min(std::max(0.0, lo), hi);
    // predictor on the Taylor model (valid near l = 0)
    auto model = [&](double l, double *mass, double *der) {
        *mass = M[0] + l * (M[1] + l * (M[2] / 2.0 + l * (M[3] / 6.0 + l * M[4] / 24.0)));
        *der = M[1] + l * (M[2] + l * (M[3] / 2.0 + l * M[4] / 6.0));
    };
    {
        const double slo = lo, shi = hi;
        double l = lam, m, d;
        model(l, &m, &d);
        for (int k = 0; k < 30 && std::fabs(m - target) > 0.01 * tol && std::fabs(l) <= 0.25; ++k) {
            if (!(d > 0.0)) break;
            const double nl_ = l - (m - target) / d;
            if (!(nl_ > slo && nl_ < shi)) break;
            l = nl_;
            model(l, &m, &d);
        }
        if (std::isfinite(l) && l > slo && l < shi && std::fabs(l) <= 0.25) lam = l;
        lo = slo; hi = shi;
    }
    double mass = 0, der = 0;
    TRY(direct(&lam, 1, &mass, &der));
    double res = mass - target;
    // |F''(l)| = |sum (1-h) sigma''| <= sum(1-h) / (6 sqrt 3): after a Newton
    // step of length d from an exactly evaluated point, |F| <= K2 d^2 / 2
    // (+ the rounding of the evaluated sum).  When that bound is below tol
    // the step is accepted without another full-grid evaluation.
    const double K2 = M[1] > 0.0 ? c->sum_alpha / (6.0 * 1.7320508075688772) : INFINITY;
    bool certified = false;
    for (int it = 0; it < P.zero_mode_max_iterations && std::fabs(res) > tol; ++it) {
        const double l0 = lam;
        update(lam, res, der);
        iters = it + 1;
        const double d = lam - l0;
        const double bound = 0.5 * K2 * d * d + 1e-14 * std::fabs(target);
        if (std::isfinite(bound) && bound <= tol && std::isfinite(der) && der > 0.0 &&
            std::fabs(res / der - (l0 - lam)) <= 1e-15 * (std::fabs(l0) + 1.0) + std::fabs(d) * 1e-12) {
            res = bound;            // reported residual: the certified bound
            certified = true;
            break;
        }
        TRY(direct(&lam, 1, &mass, &der));
        if (!std::isfinite(mass) || !std::isfinite(der)) return fail("non-finite mass");
        res = mass - target;
    }
    (void)certified;
    if (!(std::fabs(res) <= tol)) {
        TRY(check_bracket());
        return fail("did not converge");
    }
    if (ymin + lam < -P.Y_clip || ymax + lam > Ycap) return fail("shifted Y leaves [-Y_clip, Y_cap]");
    c->Yc += lam;
    c->dYoff = lam / P.dt;
    c->zm_lambda = lam;
    c->zm_residual = res;
    c->zm_derivative = der;
    c->zm_iterations = (uint64_t)iters;
    c->zm_accepted++;
    if (st) {
        st->zero_mode_iterations = iters;
        st->zero_mode_newton_steps = nwt;
        st->zero_mode_bisection_steps = bis;
        st->zero_mode_lambda = lam;
        st->zero_mode_residual = res;
        st->zero_mode_target_mass = target;
    }
    return PFGB_OK;
}

// the conservative modes' transport, before the step's elastic solve
// (main_cuda.cu:28486-28545): the context at phi^n, mu there, the six
// checkerboard sweeps (x, y, z; parity 0 then 1; their limited-face counts
// into DS_EV .. DS_EV + 5), the context again
template <typename T, typename TE>
static pfgb_status cons_transport(pfgb_ctx *c) {
    const pfgb_params &P = c->p;
    DevState<T, TE> d = dev_state<T, TE>(c);
    const ConsArgs a = cons_args(c);
    const int nb = 304;
    k_cons_context<T, TE><<<nb, 256, 0, c->stream>>>(d, a, c->cstore, d.phi_old);
    k_cons_mu<T, TE><<<nb, 256, 0, c->stream>>>(d, c->pc, c->cmu);
    PFGB_CUDA_TRY(cudaGetLastError());
    const double sp[3] = {P.dx, P.dy, P.dz};
    for (int ax = 0; ax < 3; ++ax)
        for (int par = 0; par < 2; ++par) {
            k_cons_sweep<T, TE><<<nb, 256, 0, c->stream>>>(d, c->pc, a, c->cstore, c->cmu, ax, par, sp[ax]);
            PFGB_CUDA_TRY(cudaGetLastError());
            TRY(reduce_to<AccSum1>(c, nb, DS_EV + 2 * ax + par));
        }
    k_cons_context<T, TE><<<nb, 256, 0, c->stream>>>(d, a, c->cstore, d.phi_old);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// the storage constraint on the new phi (main_cuda.cu:29859-29871): a cell
// that would leave its storage bounds, or a non-finite context, rejects the
// step (the reference's PF_CONSERVATIVE_STEP_REJECTED)
template <typename T, typename TE>
static pfgb_status cons_constrain(pfgb_ctx *c, const DevState<T, TE> &d) {
    const int nb = 304;
    k_cons_constrain<T, TE><<<nb, 256, 0, c->stream>>>(d, cons_args(c), c->cstore);
    PFGB_CUDA_TRY(cudaGetLastError());
    TRY(reduce_to<AccSum2>(c, nb, DS_BR));
    TRY(sync_read(c, DS_BR, 2));
    const double bad = c->hscal[DS_BR], capped = c->hscal[DS_BR + 1];
    TRY(sync_read(c, DS_EV, 6));
    double lim = 0.0;
    for (int i = 0; i < 6; ++i) lim += c->hscal[DS_EV + i];
    c->cons_limited = (int)(lim + 0.5);
    c->cons_constrained = (int)(capped + 0.5);
    if (bad > 0.5) {
        pfgb_set_error_msg("conservative composition step rejected at step %d: %.0f cells out of their storage "
                           "bounds or not finite", c->step + 1, bad);
        return PFGB_ERR_NONCONVERGED;
    }
    return PFGB_OK;
}

// the local redistribution of the q split's out-of-bounds transport, on
// the host as in the reference (q_transport_conservative_local_redistribution,
// main_cuda.cu:22362-22456): every cell's trial q0 + dt div J is bounded to
// [0, 1 - h]; in cell order each cell's excess (deficit) goes to the cells of
// growing Chebyshev shells around it, radius 1 to 8, periodic, in the order
// of the offsets (di, dj, dk) from -r to r, within their capacity 1 - h - q
// (storage q).  Fails when an amount stays unresolved beyond the tolerance.
static bool q_redistribute_host(int Nx, int Ny, int Nz, const std::vector<double> &q0, const std::vector<double> &divJ,
                                const std::vector<double> &phi, double dt, std::vector<double> &q, int *violating,
                                double *unresolved_out) {
    const size_t N = (size_t)Nx * Ny * Nz;
    const int R = 8;
    std::vector<double> alpha(N), res(N);
    q.assign(N, 0.0);
    int nv = 0;
    for (size_t i = 0; i < N; ++i) {
        alpha[i] = 1.0 - pf_h(clamp01(phi[i]));
        const double trial = q0[i] + dt * divJ[i];
        const double b = std::fmin(std::fmax(trial, 0.0), alpha[i]);
        q[i] = b;
        res[i] = trial - b;
        if (!std::isfinite(trial) || std::fabs(res[i]) > kQTol) ++nv;
    }
    double unresolved = 0.0;
    for (size_t i = 0; i < N; ++i) {
        double amt = res[i];
        if (!std::isfinite(amt)) { unresolved = INFINITY; continue; }
        if (std::fabs(amt) <= kQTol) continue;
        const int k0 = (int)(i % Nz), j0 = (int)((i / Nz) % Ny), i0 = (int)(i / ((size_t)Nz * Ny));
        for (int r = 1; r <= R && std::fabs(amt) > kQTol; ++r)
            for (int di = -r; di <= r && std::fabs(amt) > kQTol; ++di)
                for (int dj = -r; dj <= r && std::fabs(amt) > kQTol; ++dj)
                    for (int dk = -r; dk <= r && std::fabs(amt) > kQTol; ++dk) {
                        if (std::max(std::max(std::abs(di), std::abs(dj)), std::abs(dk)) != r) continue;
                        const size_t n = ((size_t)((i0 + di + Nx) % Nx) * Ny + (size_t)((j0 + dj + Ny) % Ny)) * Nz +
                                         (size_t)((k0 + dk + Nz) % Nz);
                        if (amt > 0.0) {
                            const double cap = alpha[n] - q[n];
                            if (cap <= 0.0) continue;
                            const double mv = std::fmin(amt, cap);
                            q[n] += mv;
                            amt -= mv;
                        } else {
                            const double av = q[n];
                            if (av <= 0.0) continue;
                            const double mv = std::fmin(-amt, av);
                            q[n] -= mv;
                            amt += mv;
                        }
                    }
        unresolved += std::fabs(amt);
    }
    *violating = nv;
    *unresolved_out = unresolved;
    return std::isfinite(unresolved) && unresolved <= kQTol * std::max(1.0, (double)nv);
}

// the q split's phase substep (main_cuda.cu:30241-30277): the storage transfer;
// where it is infeasible anywhere, the whole phi substep is rejected (phi
// returns to phi^n and q is rebuilt from it); then the bounded context
template <typename T, typename TE>
static pfgb_status q_phase(pfgb_ctx *c, const DevState<T, TE> &d, const PhysCT<T> &pc) {
    const int nb = 304;
    k_q_phase<T, TE><<<nb, 256, 0, c->stream>>>(d, pc);
    PFGB_CUDA_TRY(cudaGetLastError());
    TRY(reduce_to<AccSum1>(c, nb, DS_ZM));
    TRY(sync_read(c, DS_ZM, 1));
    c->q_rejected = c->hscal[DS_ZM] > 0.5;
    if (c->q_rejected) {
        PFGB_CUDA_TRY(cudaMemcpyAsync(d.phi_new, d.phi_old, sizeof(T) * (size_t)c->g.N, cudaMemcpyDeviceToDevice,
                                      c->stream));
        k_q_sync<T, TE><<<nb, 256, 0, c->stream>>>(d, pc, d.phi_new, 0);
        PFGB_CUDA_TRY(cudaGetLastError());
    }
    k_q_reconstruct<T, TE><<<nb, 256, 0, c->stream>>>(d, pc, d.phi_new);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// the q split's composition update after the flux divergence
// (main_cuda.cu:30648-30707, 31227-31229): explicit transport in the final z
// pass; where a cell left its bounds, the host redistribution and the bounded
// context; then q from the new composition
template <typename T, typename TE>
static pfgb_status q_transport(pfgb_ctx *c, const DevState<T, TE> &d, const PhysCT<T> &pc, double Nf) {
    int nbq = 0;
    TRY((launch_z<T, 1, 0>(c, OpQTransportZ<T, TE>{d, pc, d.S[0]}, "z_q_transport", 7.0 * Nf * sizeof(T), &nbq)));
    TRY(reduce_to<AccSum1>(c, nbq, DS_ZM));
    TRY(sync_read(c, DS_ZM, 1));
    c->q_redistributed = 0;
    const int nb = 304;
    if (c->hscal[DS_ZM] > 0.5) {
        const size_t N = (size_t)c->g.N;
        std::vector<T> hq(N), hd(N), hp(N);
        PFGB_CUDA_TRY(cudaMemcpyAsync(hq.data(), d.qb, sizeof(T) * N, cudaMemcpyDeviceToHost, c->stream));
        PFGB_CUDA_TRY(cudaMemcpyAsync(hd.data(), d.divr, sizeof(T) * N, cudaMemcpyDeviceToHost, c->stream));
        PFGB_CUDA_TRY(cudaMemcpyAsync(hp.data(), d.phi_new, sizeof(T) * N, cudaMemcpyDeviceToHost, c->stream));
        PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
        std::vector<double> q0(hq.begin(), hq.end()), dj(hd.begin(), hd.end()), ph(hp.begin(), hp.end()), qa;
        int nv = 0;
        double unresolved = 0.0;
        if (!q_redistribute_host(c->g.Nx, c->g.Ny, c->g.Nz, q0, dj, ph, c->p.dt, qa, &nv, &unresolved)) {
            pfgb_set_error_msg("q transport step rejected at step %d: %d cells out of bounds, unresolved mass %.17e",
                               c->step + 1, nv, unresolved);
            return PFGB_ERR_NONCONVERGED;
        }
        std::vector<T> hqa(qa.begin(), qa.end());
        PFGB_CUDA_TRY(cudaMemcpyAsync(d.q, hqa.data(), sizeof(T) * N, cudaMemcpyHostToDevice, c->stream));
        k_q_reconstruct<T, TE><<<nb, 256, 0, c->stream>>>(d, pc, d.phi_new);
        PFGB_CUDA_TRY(cudaGetLastError());
        PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));   // hqa is read by the copy
        c->q_redistributed = nv;
    }
    k_q_sync<T, TE><<<nb, 256, 0, c->stream>>>(d, pc, d.phi_new, c->q_redistributed ? 1 : 0);
    PFGB_CUDA_TRY(cudaGetLastError());
    return PFGB_OK;
}

// Y (composition) update: mu -> flux -> semi-implicit update -> dY/dt and
// the zero mode (main_cuda.cu:30280-30800, 31618-31623).  d.phi_old = phi^n,
// d.phi_new = phi^{n+1}; Y and the stored strain are those of the step start.
// the GP storage-coupled Y update through div J in real space: the storage
// point updates (gp_y_update_mode storage_exact / picard_storage) and the
// local_clip eta limiter (main_cuda.cu:30449-30503, 30587-30591,
// 30734-30760, 30912-30952).  Entered with the gradient of mu in real space
// (S[0..2]).  With the limiter the flux and div J are formed again with the
// limited eta and the feasibility pass runs on them once more; the
// right-hand side update then uses that div J and the final eta.  The
// reference keeps x^n for the mobility in the buffer of div J (d_xB_prev_r =
// d_divJ_r, main_cuda.cu:27858), so its second flux evaluates the mobility
// at the first pass's div J; that is reproduced unless
// gp_limiter_flux_from_xn = 1, which takes x^n.
template <typename T, typename TE>
static pfgb_status gp_y_update(pfgb_ctx *c, const DevState<T, TE> &d, pfgb_step_stats *st) {
    const pfgb_params &P = c->p;
    const PhysCT<T> pc = phys_as<T>(c->pc);
    const ElasC<TE> ec = elas_consts<TE>(c);
    const KTab kt = d.kt;
    const double invN = 1.0 / (double)c->g.N;
    const double Nf = (double)c->g.N;
    AxisIO<T, 1, 1> io1;
    io1.in[0] = d.S[0]; io1.out[0] = d.S[0];
    const bool direct = pc.gpy == 3;
    const int lim = P.gp_eta_mass_limiter == PFGB_GP_ETA_LIMITER_LOCAL_CLIP;
    const int picard = P.gp_y_update_mode == PFGB_GP_Y_PICARD_STORAGE;
    const int iters = P.gp_y_picard_iters > 0 ? P.gp_y_picard_iters : 1;
    const int passes = lim ? 2 : 1;
    const bool alias = lim && !P.gp_limiter_flux_from_xn;
    for (int pass = 0; pass < passes; ++pass) {
        if (pass == 1) {   // mu is unchanged; its gradient again for the new flux
            TRY((launch_z<T, 0, 1>(c, OpMuR2C<T, TE, true>{d, pc, ec}, "z_mu", 4.0 * Nf * sizeof(T))));
            TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
            AxisIO<T, 1, 3> iog;
            iog.in[0] = d.S[0];
            iog.out[0] = d.S[0]; iog.out[1] = d.S[1]; iog.out[2] = d.S[2];
            TRY((launch_axis<T, 1, 3, -1, +1>(c, 2, iog, OpGradX<T>{kt, invN}, "x_grad")));
            AxisIO<T, 3, 3> io3;
            for (int i = 0; i < 3; ++i) { io3.in[i] = d.S[i]; io3.out[i] = d.S[i]; }
            TRY((launch_axis<T, 3, 3, +1, 0>(c, 1, io3, OpCopy<T, 3>{}, "y_inv3")));
        }
        OpFluxZ<T, TE, true> fx{d, pc, 1, 0};
        if (pass == 1 && alias) {
            fx.xmob = d.divr;
            fx.tcd = c->pc.tc;
            const double md[6] = {P.Vm_alpha_0, P.dVm_alpha_dxB, P.Vm_compound, P.D_alpha, P.gp_M_GP, P.gp_M_beta};
            for (int i = 0; i < 6; ++i) fx.md[i] = md[i];
        }
        TRY((launch_z<T, 3, 5>(c, fx, "z_flux", 5.0 * Nf * sizeof(T))));
        {
            AxisIO<T, 4, 3> io;
            for (int i = 0; i < 4; ++i) io.in[i] = d.S[i];
            io.out[0] = d.S[0]; io.out[1] = d.S[1]; io.out[2] = d.S[3];
            TRY((launch_axis<T, 4, 3, -1, 0>(c, 1, io, OpYCombY<T>{kt}, "y_ycomb")));
        }
        {
            AxisIO<T, 2, 1> io;
            io.in[0] = d.S[0]; io.in[1] = d.S[1];
            io.out[0] = d.S[0];
            TRY((launch_axis<T, 2, 1, -1, +1>(c, 2, io, OpDivX<T>{kt, invN}, "x_div")));
        }
        TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
        const int stage = (pass + 1 < passes) ? 0 : (direct ? 1 : 2);
        int nb = 0;
        OpGPEtaZ<T, TE> ge{d, pc, d.S[0], lim, stage, picard, iters, invN};
        ge.keep_div = stage == 0 && alias;
        TRY((launch_z<T, 1, 0>(c, ge, "z_gp_eta", (stage == 1 ? 9.0 : 7.0) * Nf * sizeof(T), &nb)));
        TRY(reduce_to<AccSum2>(c, nb, DS_BR + 2 * pass));
    }
    const double *meanDY = c->dscal + DS_BR + 2 * (passes - 1) + 1;
    if (!direct) {
        TRY((launch_z<T, 0, 2>(c, OpGPRhsZ<T, TE>{d, pc}, "z_gp_rhs", 8.0 * Nf * sizeof(T))));
        AxisIO<T, 2, 2> io2;
        for (int i = 0; i < 2; ++i) { io2.in[i] = d.S[i]; io2.out[i] = d.S[i]; }
        TRY((launch_axis<T, 2, 2, -1, 0>(c, 1, io2, OpCopy<T, 2>{}, "y_fwd2")));
        AxisIO<T, 2, 1> iox;
        iox.in[0] = d.S[0]; iox.in[1] = d.S[1];
        iox.out[0] = d.S[0];
        TRY((launch_axis<T, 2, 1, -1, +1>(c, 2, iox, OpYUpdRX<T>{kt, P.dt, invN, meanDY}, "x_y_update")));
        TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
        int nbf = 0;
        TRY((launch_z<T, 1, 0>(c, OpYFinalZ<T, TE>{d, pc, d.S[0]}, "z_y_final", 4.0 * Nf * sizeof(T), &nbf)));
    }
    c->dYoff = 0.0;
    c->gp_limited = 0;
    if (st) {
        TRY(sync_read(c, DS_BR, 4));
        c->gp_limited = (int)(c->hscal[DS_BR] + (lim ? c->hscal[DS_BR + 2] : 0.0) + 0.5);
        st->mean_DY = c->hscal[DS_BR + 2 * (passes - 1) + 1];
    }
    return PFGB_OK;
}

template <typename T, typename TE>
static pfgb_status y_update(pfgb_ctx *c, const DevState<T, TE> &d, pfgb_step_stats *st) {
    const pfgb_params &P = c->p;
    const PhysCT<T> pc = phys_as<T>(c->pc);
    const ElasC<TE> ec = elas_consts<TE>(c);
    const KTab kt = d.kt;
    const double invN = 1.0 / (double)c->g.N;
    const double Nf = (double)c->g.N;
    AxisIO<T, 1, 1> io1;
    io1.in[0] = d.S[0]; io1.out[0] = d.S[0];
    int nb = 0;
    const double mu_bytes = (3.0 + pc.gp) * Nf * sizeof(T) + (pc.elastic ? 6.0 : 0.0) * Nf * sizeof(TE);
    if (pc.gpy)
        TRY((launch_z<T, 0, 1>(c, OpMuR2C<T, TE, true>{d, pc, ec}, "z_mu", mu_bytes + Nf * sizeof(T), &nb)));
    else
        TRY((launch_z<T, 0, 1>(c, OpMuR2C<T, TE>{d, pc, ec}, "z_mu", mu_bytes, &nb)));
    TRY(reduce_to<AccSum1>(c, nb, DS_MEAN_DY, invN));
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
    {
        AxisIO<T, 1, 3> io;
        io.in[0] = d.S[0];
        io.out[0] = d.S[0]; io.out[1] = d.S[1]; io.out[2] = d.S[2];
        TRY((launch_axis<T, 1, 3, -1, +1>(c, 2, io, OpGradX<T>{kt, invN}, "x_grad")));
    }
    {
        AxisIO<T, 3, 3> io;
        for (int i = 0; i < 3; ++i) { io.in[i] = d.S[i]; io.out[i] = d.S[i]; }
        TRY((launch_axis<T, 3, 3, +1, 0>(c, 1, io, OpCopy<T, 3>{}, "y_inv3")));
    }
    // GP storage coupling with a storage point update or the eta limiter
    if (pc.gpy == 3 || (pc.gpy && P.gp_eta_mass_limiter == PFGB_GP_ETA_LIMITER_LOCAL_CLIP))
        return gp_y_update<T, TE>(c, d, st);
    const bool storage_exact = P.pf_y_update_mode == PFGB_Y_STORAGE_EXACT;
    const bool qsplit = P.pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT;
    const bool divj_real = storage_exact || qsplit || P.pf_y_update_mode == PFGB_Y_X_TRANSPORT_SPLIT;
    if (pc.gpy)
        TRY((launch_z<T, 3, 5>(c, OpFluxZ<T, TE, true>{d, pc, 0, 0}, "z_flux", 6.0 * Nf * sizeof(T))));
    else
        TRY((launch_z<T, 3, 5>(c, OpFluxZ<T, TE>{d, pc, divj_real ? 1 : 0, qsplit ? 1 : 0}, "z_flux",
                               (4.0 + pc.gp) * Nf * sizeof(T))));
    if (divj_real) {
        {
            AxisIO<T, 4, 3> io;
            for (int i = 0; i < 4; ++i) io.in[i] = d.S[i];
            io.out[0] = d.S[0]; io.out[1] = d.S[1]; io.out[2] = d.S[3];
            TRY((launch_axis<T, 4, 3, -1, 0>(c, 1, io, OpYCombY<T>{kt}, "y_ycomb")));
        }
        {
            AxisIO<T, 2, 1> io;
            io.in[0] = d.S[0]; io.in[1] = d.S[1];
            io.out[0] = d.S[0];
            TRY((launch_axis<T, 2, 1, -1, +1>(c, 2, io, OpDivX<T>{kt, invN}, "x_div")));
        }
        TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
        if (storage_exact) {
            TRY((launch_z<T, 1, 0>(c, OpStorageExactZ<T, TE>{d, pc, d.S[0], P.gp_h_alpha_eps}, "z_storage_exact",
                                   5.0 * Nf * sizeof(T))));
        } else if (qsplit) {
            TRY((q_transport<T, TE>(c, d, pc, Nf)));
        } else {
            const double mDx = P.D_alpha * P.pf_composition_stabilizer_Dalpha_multiplier;
            TRY((launch_z<T, 1, 2>(c, OpXSplitSrcZ<T, TE>{d, pc, P.pf_matrix_storage_floor}, "z_xsplit_src",
                                   2.0 * Nf * sizeof(T))));
            AxisIO<T, 2, 2> io2;
            for (int i = 0; i < 2; ++i) { io2.in[i] = d.S[i]; io2.out[i] = d.S[i]; }
            TRY((launch_axis<T, 2, 2, -1, 0>(c, 1, io2, OpCopy<T, 2>{}, "y_fwd2")));
            AxisIO<T, 2, 1> iox;
            iox.in[0] = d.S[0]; iox.in[1] = d.S[1];
            iox.out[0] = d.S[0];
            TRY((launch_axis<T, 2, 1, -1, +1>(c, 2, iox, OpXSplitX<T>{kt, P.dt, invN, mDx}, "x_xsplit")));
            TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
            TRY((launch_z<T, 1, 0>(c, OpXSplitFinalZ<T, TE>{d, pc, d.S[0]}, "z_xsplit_final", 4.0 * Nf * sizeof(T))));
        }
        c->dYoff = 0.0;
        if (st) {
            if (storage_exact) {
                TRY(sync_read(c, DS_MEAN_DY, 1));
                st->mean_DY = c->hscal[DS_MEAN_DY];
            } else {
                st->mean_DY = P.D_alpha * P.pf_composition_stabilizer_Dalpha_multiplier;
            }
        }
        return PFGB_OK;
    }
    {
        AxisIO<T, 4, 3> io;
        for (int i = 0; i < 4; ++i) io.in[i] = d.S[i];
        io.out[0] = d.S[0]; io.out[1] = d.S[1]; io.out[2] = d.S[3];
        TRY((launch_axis<T, 4, 3, -1, 0>(c, 1, io, OpYCombY<T>{kt}, "y_ycomb")));
    }
    {
        AxisIO<T, 3, 1> io;
        io.in[0] = d.S[0]; io.in[1] = d.S[1]; io.in[2] = d.S[3];
        io.out[0] = d.S[0];
        TRY((launch_axis<T, 3, 1, -1, +1>(c, 2, io, OpYUpdX<T>{kt, P.dt, invN, c->dscal + DS_MEAN_DY}, "x_y_update")));
    }
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
    int nbf = 0;
    TRY((launch_z<T, 1, 0>(c, OpYFinalZ<T, TE>{d, pc, d.S[0]}, "z_y_final", (4.0 + pc.zm) * Nf * sizeof(T), &nbf)));
    c->dYoff = 0.0;
    if (P.zero_mode_enabled) TRY((zero_mode<T, TE>(c, nbf, st)));
    if (st) {
        if (!P.zero_mode_enabled) TRY(sync_read(c, DS_MEAN_DY, 1));
        st->mean_DY = c->hscal[DS_MEAN_DY];
    }
    return PFGB_OK;
}

template <typename T, typename TE>
static pfgb_status step_once(pfgb_ctx *c, pfgb_step_stats *st) {
    using T2 = cplx_t<T>;
    const pfgb_params &P = c->p;
    const PhysCT<T> pc = phys_as<T>(c->pc);
    const ElasC<TE> ec = elas_consts<TE>(c);
    c->Yc_prev = c->Yc;
    // conservative composition modes: the transport before the elastic solve
    const bool cons = P.pf_composition_mode != PFGB_COMPOSITION_LEGACY;
    c->cons_limited = c->cons_constrained = 0;
    if (cons) TRY((cons_transport<T, TE>(c)));
    if (P.elastic_enabled) TRY((elastic_solve<T, TE>(c, st)));
    DevState<T, TE> d = dev_state<T, TE>(c);
    const KTab kt = d.kt;
    const double invN = 1.0 / (double)c->g.N;
    const double Nf = (double)c->g.N;
    AxisIO<T, 1, 1> io1;
    io1.in[0] = d.S[0]; io1.out[0] = d.S[0];

    // ---- phi ----
    TRY((launch_z<T, 0, 1>(c, OpPhiR2C<T, TE>{d, pc, ec}, "z_phi_rhs", (2.0 + pc.gp) * Nf * sizeof(T) + (pc.coupling ? 6.0 : 0.0) * Nf * sizeof(TE))));
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
    TRY((launch_axis<T, 1, 1, -1, +1>(c, 2, io1, OpACFilterX<T>{kt, P.L_phi * P.dt * P.kappa_phi, invN}, "x_ac_filter")));
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
    TRY((launch_z<T, 1, 0>(c, OpACStoreZ<T, TE>{d.S[0], d.phi_new, c->g.NzC, T(-1e-6), T(1.0 + 1e-6)}, "z_ac_store", Nf * sizeof(T))));
    if (cons) TRY((cons_constrain<T, TE>(c, d)));

    // ---- eta (GP zone) ----
    if (pc.gp) {
        TRY((launch_z<T, 0, 1>(c, OpEtaR2C<T, TE>{d, pc, ec}, "z_eta_rhs", 3.0 * Nf * sizeof(T))));
        TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
        TRY((launch_axis<T, 1, 1, -1, +1>(c, 2, io1, OpACFilterX<T>{kt, P.gp_L_eta * P.dt * P.gp_kappa_eta, invN}, "x_ac_filter")));
        TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
        TRY((launch_z<T, 1, 0>(c, OpACStoreZ<T, TE>{d.S[0], d.eta_new, c->g.NzC, T(0), T(1)}, "z_ac_store", Nf * sizeof(T))));
    }

    // q split: the phase substep's storage transfer
    c->q_rejected = 0;
    if (P.pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT) TRY((q_phase<T, TE>(c, d, pc)));

    // the conservative modes carry the composition in their storage: no Y
    // update and no dY/dt update (main_cuda.cu:30283-30284)
    if (!cons) TRY((y_update<T, TE>(c, d, st)));
    if (st) {
        st->q_phase_rejected = c->q_rejected;
        st->q_redistributed_cells = c->q_redistributed;
        st->cons_limited_faces = c->cons_limited;
        st->gp_eta_limited_cells = c->gp_limited;
        st->cons_phase_constrained = c->cons_constrained;
    }
    c->cur = 1 - c->cur;
    if (pc.gp) c->ecur = 1 - c->ecur;
    c->step++;
    (void)sizeof(T2);
    return PFGB_OK;
}

// ===========================================================================
// minimize (mode = minimize, full model, two_phase): gradient flow of phi
// with the Lagrange volume multiplier, the Y update, post-projection and the
// V0 projection (main_cuda.cu:29264-29750, 32100-32600)
// ===========================================================================
// z pass producer: explicit drive g_e at phi (stored in mge; stress frozen
// at the iteration's elastic solve) and phi itself -> R2C for Lap(phi)
template <typename T, typename TE>
struct OpMinGradZ {
    using Acc = NoAcc;
    DevState<T, TE> d; PhysCT<T> c; ElasC<TE> ec; const T *phi;
    int phi_only;   // minimize_full_model = 0: compute_phi_rhs_minimize_kernel
    __device__ void point(long long cell, const T *, T *out, Acc &) const {
        const T p = phi[cell];
        TE e[6], sg[6];
        if (c.coupling) {
#pragma unroll
            for (int a = 0; a < 6; ++a) { e[a] = d.eps[a][cell]; sg[a] = d.sig[a][cell]; }
        }
        if (phi_only) {
            d.mge[cell] = phi_rhs_phi_only<T, TE>(c, ec, p, e, sg);
        } else {
            const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
            d.mge[cell] = phi_rhs_sig<T, TE>(c, ec, p, c.gp ? d.eta_old[cell] : T(0), xB, e, sg);
        }
        out[0] = p;
    }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        d.S[0][row * d.g.NzC + k] = v[0];
    }
};

// x pass: Lap = mask (-k^2) mask phi_k / N (compute_laplacian_k_kernel)
template <typename T>
struct OpLapX {
    static constexpr bool kInplace = false;
    KTab kt; double invN;
    __device__ void apply(int i, int j, int k, const cplx_t<T> *in, cplx_t<T> *out) const {
        if (kt.cut(i, j, k)) { out[0] = mk2<cplx_t<T>>(T(0), T(0)); return; }
        out[0] = cscale(in[0], T(-kt.k2(i, j, k) * invN));
    }
};

// z pass consumer: store Lap(phi); sums of h'(phi) g_full and h'(phi)^2 with
// g_full = g_e - kappa Lap (the volume multiplier, :29484-29489)
template <typename T, typename TE>
struct OpMinLapZ {
    using Acc = AccSum2;
    DevState<T, TE> d; const T *phi; double kappa;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = d.S[0][row * d.g.NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &acc) const {
        const T lap = in[0];
        d.mlap[cell] = lap;
        const T gf = d.mge[cell] - T(kappa) * lap;
        const T hp = pf_hp(phi[cell]);
        acc.a += double(hp * gf);
        acc.b += double(hp * hp);
    }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
    __device__ void finish(int b, const Acc &a) const { reinterpret_cast<Acc *>(d.partials)[b] = a; }
};

// z pass producer of the constrained step: phi - L dt [(g_full + kappa Lap) + lambda h']
template <typename T, typename TE>
struct OpMinStepR2C {
    using Acc = NoAcc;
    DevState<T, TE> d; const T *phi; double kappa, Ldt, lambda;
    __device__ void point(long long cell, const T *, T *out, Acc &) const {
        const T p = phi[cell];
        const T lap = d.mlap[cell];
        const T gf = d.mge[cell] - T(kappa) * lap;
        const T r = (gf - T(-kappa) * lap) + T(lambda) * pf_hp(p);
        out[0] = p - T(Ldt) * r;
    }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const {
        d.S[0][row * d.g.NzC + k] = v[0];
    }
};

// energies of the iteration start (:29264-29345): <h>, gradient energy by
// central differences, double well, elastic energy density and its h-weighted
// sum (compute_gel_density_kernel), chemical excess (compute_gbulk_excess_hat)
struct AccMinE {
    static constexpr bool kActive = true;
    double mh, grad, dw, gel, gelh, chem;
    __device__ static AccMinE identity() { return {0, 0, 0, 0, 0, 0}; }
    __device__ static AccMinE combine(AccMinE a, const AccMinE &b) {
        a.mh += b.mh; a.grad += b.grad; a.dw += b.dw; a.gel += b.gel; a.gelh += b.gelh; a.chem += b.chem;
        return a;
    }
    __device__ static AccMinE shfl_down(AccMinE a, int o) {
        AccMinE r;
        double *pa = reinterpret_cast<double *>(&a), *pr = reinterpret_cast<double *>(&r);
#pragma unroll
        for (int i = 0; i < 6; ++i) pr[i] = __shfl_down_sync(0xffffffffu, pa[i], o);
        return r;
    }
};

template <typename T, typename TE>
__global__ void __launch_bounds__(256)
k_min_energy(DevState<T, TE> d, PhysC c, ElasC<TE> ec, const T *phi, double g0, int chem, AccMinE *part) {
    AccMinE a = AccMinE::identity();
    const int Nx = d.g.Nx, Ny = d.g.Ny, Nz = d.g.Nz;
    const double idx2 = 0.5 / c.dx, idy2 = 0.5 / c.dy, idz2 = 0.5 / c.dz;
    for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < d.g.N;
         cell += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(cell % Nz);
        const long long r = cell / Nz;
        const int j = (int)(r % Ny), i = (int)(r / Ny);
        const int ip = i + 1 == Nx ? 0 : i + 1, im = i == 0 ? Nx - 1 : i - 1;
        const int jp = j + 1 == Ny ? 0 : j + 1, jm = j == 0 ? Ny - 1 : j - 1;
        const int kp = k + 1 == Nz ? 0 : k + 1, km = k == 0 ? Nz - 1 : k - 1;
        const double gx = (double(phi[((long long)ip * Ny + j) * Nz + k]) - double(phi[((long long)im * Ny + j) * Nz + k])) * idx2;
        const double gy = (double(phi[((long long)i * Ny + jp) * Nz + k]) - double(phi[((long long)i * Ny + jm) * Nz + k])) * idy2;
        const double gz = (double(phi[r * Nz + kp]) - double(phi[r * Nz + km])) * idz2;
        const T p = phi[cell];
        a.grad += 0.5 * c.kappa * (gx * gx + gy * gy + gz * gz);
        a.dw += c.W * double(pf_g(p));
        const T h = pf_h(clamp01(p));
        a.mh += double(h);
        // the monitor's composition: sigmoid(Y), capped once clamped
        const T xB = xB_of_Y<T>(c, d.Y[cell] + T(d.Yc));
        const T xm = xB < T(c.xbcap) ? xB : T(c.xbcap);
        if (c.elastic) {
            TE e0[6];
            eigenstrain<T, TE>(c, ec, p, c.gp ? d.eta_old[cell] : T(0), clamp01(xm), c.gp_el != 0, e0);
            double sd = 0.0;
#pragma unroll
            for (int q = 0; q < 6; ++q)
                sd += (q < 3 ? 1.0 : 2.0) * double(d.sig[q][cell]) * (double(d.eps[q][cell]) - double(e0[q]));
            a.gel += 0.5 * sd;
            a.gelh += 0.5 * sd * double(h);
        }
        if (chem) {
            const T x = clamp_eps(xm, T(1e-12));
            T offA, offB;
            thermo_mu_off<T>(c.tc, x, offA, offB);
            const double mix = (1.0 - double(x)) * (c.tc.GA_s + double(offA)) + double(x) * (c.tc.GB_s + double(offB));
            a.chem += (1.0 - double(h)) * mix + double(h) * c.mu0 - g0;
        }
    }
    block_reduce_acc(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// projected KKT residual (:684-708) with the exact multiplier, and |phi - phi^n|^2
template <typename T, typename TE>
__global__ void __launch_bounds__(256)
k_min_resid(DevState<T, TE> d, const T *phi, const T *phin, double kappa, double lk, AccSum2 *part) {
    AccSum2 a = AccSum2::identity();
    for (long long cell = blockIdx.x * (long long)blockDim.x + threadIdx.x; cell < d.g.N;
         cell += (long long)gridDim.x * blockDim.x) {
        const T p = phi[cell];
        T rr = (d.mge[cell] - T(kappa) * d.mlap[cell]) + T(lk) * pf_hp(p);
        if ((p <= T(1e-12) && rr > T(0)) || (p >= T(1) - T(1e-12) && rr < T(0))) rr = T(0);
        a.a += double(rr) * double(rr);
        const double dp = double(p) - double(phin[cell]);
        a.b += dp * dp;
    }
    block_reduce_acc(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// sum h(clamp01 phi) and sum h'(phi)^2 (gpu_compute_vf_from_h, :5609; hprime_sq)
template <typename T>
__global__ void __launch_bounds__(256)
k_min_hsums(const T *phi, long long N, AccSum2 *part) {
    AccSum2 a = AccSum2::identity();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const T p = phi[i];
        a.a += double(pf_h(clamp01(p)));
        const T hp = pf_hp(p);
        a.b += double(hp * hp);
    }
    block_reduce_acc(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

// apply_volume_projection_kernel (:636-645)
template <typename T>
__global__ void k_min_project(T *phi, long long N, double lc) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const T p = phi[i];
        phi[i] = clamp01(p + T(lc) * pf_hp(p));
    }
}

// |Y - Y^n|^2 and the largest xB (the monitor's safety clamp test)
struct AccSumMax {
    static constexpr bool kActive = true;
    double s, m;
    __device__ static AccSumMax identity() { return {0.0, -1e300}; }
    __device__ static AccSumMax combine(AccSumMax a, AccSumMax b) { return {a.s + b.s, fmax(a.m, b.m)}; }
    __device__ static AccSumMax shfl_down(AccSumMax x, int o) {
        return {__shfl_down_sync(0xffffffffu, x.s, o), __shfl_down_sync(0xffffffffu, x.m, o)};
    }
};
template <typename T, typename TE>
__global__ void __launch_bounds__(256)
k_min_dy(DevState<T, TE> d, PhysCT<T> c, double yc_prev, AccSumMax *part) {
    AccSumMax a = AccSumMax::identity();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < d.g.N;
         i += (long long)gridDim.x * blockDim.x) {
        const double y = double(d.Y[i]) + d.Yc, yp = double(d.Yprev[i]) + yc_prev;
        a.s += (y - yp) * (y - yp);
        a.m = fmax(a.m, double(xB_of_Y<T>(c, T(y))));
    }
    block_reduce_acc(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

static const int kMinBlocks = 1216;   // 8 x 152 SMs

// Lap(phi), g_e and the multiplier sums at `phi`; returns -sum h'g / sum h'^2
template <typename T, typename TE>
static pfgb_status min_gradient(pfgb_ctx *c, const DevState<T, TE> &d, const T *phi, double *lambda) {
    const double invN = 1.0 / (double)c->g.N, Nf = (double)c->g.N;
    const ElasC<TE> ec = elas_consts<TE>(c);
    AxisIO<T, 1, 1> io1;
    io1.in[0] = d.S[0]; io1.out[0] = d.S[0];
    TRY((launch_z<T, 0, 1>(c, OpMinGradZ<T, TE>{d, phys_as<T>(c->pc), ec, phi, !c->p.minimize_full_model}, "z_min_grad",
                           3.0 * Nf * sizeof(T) + (c->pc.coupling ? 12.0 : 0.0) * Nf * sizeof(TE))));
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
    TRY((launch_axis<T, 1, 1, -1, +1>(c, 2, io1, OpLapX<T>{d.kt, invN}, "x_lap")));
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
    int nb = 0;
    TRY((launch_z<T, 1, 0>(c, OpMinLapZ<T, TE>{d, phi, c->p.kappa_phi}, "z_min_lap", 3.0 * Nf * sizeof(T), &nb)));
    TRY(reduce_to<AccSum2>(c, nb, 40));
    TRY(sync_read(c, 40, 2));
    const double shg = c->hscal[40], sh2 = c->hscal[41];
    *lambda = std::fabs(sh2) > 1e-30 ? -shg / sh2 : 0.0;
    return PFGB_OK;
}

// semi-implicit constrained step from `src` into `dst` (the reference's
// phi_semi_implicit_update + dealias + Z2D + normalize_and_clamp)
template <typename T, typename TE>
static pfgb_status min_step(pfgb_ctx *c, const DevState<T, TE> &d, const T *src, T *dst, double lambda) {
    const pfgb_params &P = c->p;
    const double invN = 1.0 / (double)c->g.N, Nf = (double)c->g.N;
    AxisIO<T, 1, 1> io1;
    io1.in[0] = d.S[0]; io1.out[0] = d.S[0];
    TRY((launch_z<T, 0, 1>(c, OpMinStepR2C<T, TE>{d, src, P.kappa_phi, P.L_phi * P.dt, lambda}, "z_min_step",
                           3.0 * Nf * sizeof(T))));
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_fwd1")));
    TRY((launch_axis<T, 1, 1, -1, +1>(c, 2, io1, OpACFilterX<T>{d.kt, P.L_phi * P.dt * P.kappa_phi, invN}, "x_ac_filter")));
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io1, OpCopy<T, 1>{}, "y_inv1")));
    TRY((launch_z<T, 1, 0>(c, OpACStoreZ<T, TE>{d.S[0], dst, c->g.NzC, T(-1e-6), T(1.0 + 1e-6)}, "z_ac_store", Nf * sizeof(T))));
    return PFGB_OK;
}

template <typename Acc, typename K, typename... A>
static pfgb_status min_reduce(pfgb_ctx *c, const char *tag, double bytes, int slot, int n, K kern, A... args) {
    {
        ProfScope ps(c, {tag, bytes});
        kern<<<kMinBlocks, 256, 0, c->stream>>>(args..., (Acc *)c->partials);
        PFGB_CUDA_TRY(cudaGetLastError());
    }
    TRY(reduce_to<Acc>(c, kMinBlocks, slot));
    TRY(sync_read(c, slot, n));
    return PFGB_OK;
}

template <typename T, typename TE>
static pfgb_status minimize_once(pfgb_ctx *c, pfgb_min_stats *ms) {
    const pfgb_params &P = c->p;
    const double Nf = (double)c->g.N;
    const long long N = c->g.N;
    // phi-only minimize (minimize_full_model = 0) carries no composition
    // (main_cuda.cu:27208-27217): its elastic solve, stress and energies use
    // the phi-only eigenstrain h(phi) eps00 (main_cuda.cu:28816-28824 and
    // the NULL xB of :28920, :29303), which is the composition cap at 0
    const bool phi_only = !P.minimize_full_model;
    c->pc.xbcap = phi_only ? 0.0 : (c->xb_clamp ? P.minimize_xB_max_safe : 2.0);
    c->Yc_prev = c->Yc;
    pfgb_step_stats st;
    memset(&st, 0, sizeof(st));
    if (P.elastic_enabled) TRY((elastic_solve<T, TE>(c, &st)));
    const int it = ++c->min_iter;
    const PhysCT<T> pc = phys_as<T>(c->pc);
    const ElasC<TE> ec = elas_consts<TE>(c);
    DevState<T, TE> d = dev_state<T, TE>(c);
    T *pa = (T *)c->phi[c->cur], *pb = (T *)c->phi[1 - c->cur];

    // ---- energies of the iteration start ----
    // reference state of the chemical excess (main_cuda.cu:27400-27431)
    const double xref = P.ic_23d_xB_out;
    double oA, oB;
    thermo_mu_off<double>(c->pc.tc, xref, oA, oB);
    const double muAr = c->pc.tc.GA_s + oA, muBf = c->pc.tc.GB_s + oB;
    const double g0 = (1.0 - xref) * muAr + xref * muBf;
    TRY((min_reduce<AccMinE>(c, "min_energy", (2.0 * Nf) * sizeof(T) + 12.0 * Nf * sizeof(TE), 42, 6,
                             k_min_energy<T, TE>, d, c->pc, ec, (const T *)pa, g0, phi_only ? 0 : 1)));
    const double *E = c->hscal + 42;
    double mean_h = E[0] / Nf;
    if (it == 1 && !(c->V0_target > 0.0)) {
        if (P.ic_phi_seed_radius > 0.0) {   // compute_effective_vf_target, :2459-2490 (spherical seeds)
            double vf = std::fmin(0.999, std::fmax(1e-6, P.ic_vf_target_phi));
            const int ns = P.ic_phi_num_seeds > 0 ? P.ic_phi_num_seeds : 1;
            const double R = P.ic_phi_seed_radius;
            const double Lx = P.Nx * P.dx, Ly = P.Ny * P.dy, Lz = P.Nz * P.dz;
            if (P.Ny > 2) { if (Lx * Ly * Lz > 0.0) vf = ns * (4.0 * PFGB_PI / 3.0) * R * R * R / (Lx * Ly * Lz); }
            else if (Lx * Lz > 0.0) vf = ns * PFGB_PI * R * R / (Lx * Lz);
            c->V0_target = vf;
        } else {
            c->V0_target = mean_h;
        }
    }
    const double total_interface = E[1] + E[2];
    const double F_surf = total_interface / Nf;
    const double F_el = P.elastic_enabled ? E[3] / Nf : 0.0;
    const double total_el_core = P.elastic_enabled ? E[4] : 0.0;
    // the chemical excess and the CNT summary are full-model only
    // (main_cuda.cu:29322-29343); NaN in phi-only minimize, and so is the
    // total, which disables the energy-plateau test there
    const double F_chem = phi_only ? NAN : E[5] / Nf;
    const double F_total = phi_only ? NAN : F_chem + F_surf + F_el;
    const double F_chem_cnt = (!phi_only && mean_h > 0.0) ? mean_h * (P.mu0_compound - muBf) : NAN;
    const double F_total_cnt = phi_only ? NAN : F_surf + F_el + F_chem_cnt;
    const double F_prev = c->prev_F_total;
    c->prev_F_total = F_total;

    // ---- phi step with the under-relaxed multiplier: pa = phi^n -> pb ----
    double eta_r = std::min(1.0, std::max(0.0, P.eta_lambda_vol));
    double lraw = 0.0;
    TRY((min_gradient<T, TE>(c, d, pa, &lraw)));
    c->lambda_vol = (1.0 - eta_r) * c->lambda_vol + eta_r * lraw;
    TRY((min_step<T, TE>(c, d, pa, pb, c->lambda_vol)));

    // ---- projected KKT residual and rms_dphi at phi^{n+1} ----
    double lk = 0.0;
    TRY((min_gradient<T, TE>(c, d, pb, &lk)));
    TRY((min_reduce<AccSum2>(c, "min_resid", 4.0 * Nf * sizeof(T), 44, 2, k_min_resid<T, TE>, d, (const T *)pb,
                             (const T *)pa, P.kappa_phi, lk)));
    const double rms_res = std::sqrt(c->hscal[44] / Nf);
    const double rms_dphi = std::sqrt(c->hscal[45] / Nf) / P.dt;

    // ---- Y update (full model only, main_cuda.cu:30284) with phi^n = pa, phi^{n+1} = pb ----
    if (!phi_only) {
        DevState<T, TE> dy = d;
        dy.phi_old = pa;
        dy.phi_new = pb;
        dy.eta_new = dy.eta_old;   // eta does not evolve in minimize (gp_zone)
        TRY((y_update<T, TE>(c, dy, &st)));
    }
    d = dev_state<T, TE>(c);   // same buffers, updated scalars
    T *cur = pb, *oth = pa;

    // ---- post-projection substeps (elastic frozen, eta = 1) ----
    for (int k = 0; k < P.minimize_post_projection_iters; ++k) {
        double l = 0.0;
        TRY((min_gradient<T, TE>(c, d, cur, &l)));
        c->lambda_vol = l;
        TRY((min_step<T, TE>(c, d, cur, oth, l)));
        std::swap(cur, oth);
    }
    TRY((min_reduce<AccSum2>(c, "min_hsums", Nf * sizeof(T), 46, 2, k_min_hsums<T>, (const T *)cur, N)));
    mean_h = c->hscal[46] / Nf;

    // ---- first-order projection of <h> onto V0 ----
    if (c->V0_target > 1e-30 && std::isfinite(mean_h)) {
        const double vol_err = c->V0_target - mean_h;
        if (std::fabs(vol_err) > 1e-14) {
            const double mhp2 = c->hscal[47] / Nf;
            const double lc = mhp2 > 1e-30 ? vol_err / mhp2 : 0.0;
            {
                ProfScope ps(c, {"min_project", 2.0 * Nf * sizeof(T)});
                k_min_project<T><<<kMinBlocks, 256, 0, c->stream>>>(cur, N, lc);
                PFGB_CUDA_TRY(cudaGetLastError());
            }
            TRY((min_reduce<AccSum2>(c, "min_hsums", Nf * sizeof(T), 46, 2, k_min_hsums<T>, (const T *)cur, N)));
            mean_h = c->hscal[46] / Nf;
        }
    }
    c->cur = cur == (T *)c->phi[0] ? 0 : 1;

    // ---- stopping rule (:32405-32600) and the monitor's xB clamp ----
    // rms_dY and the xB monitor are full-model only (NaN / off in phi-only
    // minimize, main_cuda.cu:32425-32440, 25262)
    double rms_dY = NAN, xmax = 0.0;
    if (!phi_only) {
        TRY((min_reduce<AccSumMax>(c, "min_dy", 2.0 * Nf * sizeof(T), 48, 2, k_min_dy<T, TE>, d, phys_as<T>(c->pc),
                                   c->Yc_prev)));
        rms_dY = std::sqrt(c->hscal[48] / Nf) / P.dt;
        xmax = c->hscal[49];
    }
    double edr = NAN;
    if (std::isfinite(F_prev) && std::isfinite(F_total)) edr = std::fabs(F_total - F_prev) / std::fmax(std::fabs(F_prev), 1e-20);
    const double ver = c->V0_target > 1e-30 ? std::fabs(mean_h - c->V0_target) / (c->V0_target + 1e-30) : 0.0;
    const bool vol_ok = std::isfinite(ver) && ver < P.minimize_vol_err_rel_threshold;
    const bool res_ok = std::isfinite(rms_res) && rms_res < P.minimize_rms_res_threshold;
    int condA, condB;
    if (phi_only) {   // main_cuda.cu:32541-32550: phi convergence and the energy plateau
        condA = std::isfinite(rms_dphi) && rms_dphi < P.minimize_rms_dphi_threshold && res_ok && vol_ok;
        condB = std::isfinite(edr) && edr < P.minimize_energy_diff_rel_threshold && std::isfinite(rms_dphi) &&
                rms_dphi < 5.0 * P.minimize_rms_dphi_threshold && res_ok && vol_ok;
    } else {
        condA = std::isfinite(rms_dphi) && std::isfinite(rms_dY) && rms_dphi < P.minimize_rms_dphi_threshold &&
                rms_dY < P.minimize_rms_dY_threshold && res_ok && vol_ok;
        condB = std::isfinite(edr) && edr < P.minimize_energy_diff_rel_threshold && std::isfinite(rms_dphi) &&
                std::isfinite(rms_dY) && rms_dphi < 5.0 * P.minimize_rms_dphi_threshold &&
                rms_dY < 5.0 * P.minimize_rms_dY_threshold && res_ok && vol_ok;
    }
    const double pt = (double)it * P.dt;
    const bool pt_ok = std::isfinite(pt) && pt + 1e-14 >= P.minimize_min_pseudo_time;
    c->conv_count = ((condA || condB) && pt_ok) ? c->conv_count + 1 : 0;
    if (c->conv_count >= P.minimize_convergence_steps && !c->converged_iter) c->converged_iter = it;
    // the reference clamps its stored xB when the monitor sees max xB above
    // minimize_xB_max_safe; the clamped xB is what the next iteration's
    // elastic solve and energies read (here: the cap on the elastic side)
    const int clamped = !phi_only && xmax > P.minimize_xB_max_safe + 1e-12;
    c->xb_clamp = clamped;
    c->step++;
    if (ms) {
        ms->iteration = it;
        ms->converged = c->converged_iter != 0;
        ms->converged_iteration = c->converged_iter;
        ms->convergence_count = c->conv_count;
        ms->condA = condA; ms->condB = condB;
        ms->xB_clamped = clamped;
        ms->elastic_iterations = st.elastic_iterations;
        ms->elastic_relative_residual = st.elastic_relative_residual;
        ms->mean_h = mean_h; ms->V0_target = c->V0_target; ms->lambda_vol = c->lambda_vol;
        ms->F_surf = F_surf; ms->F_el = F_el; ms->F_chem_excess = F_chem; ms->F_total_excess = F_total;
        ms->F_chem_CNT = F_chem_cnt; ms->F_total_CNT = F_total_cnt;
        ms->total_interface_sum = total_interface; ms->total_el_core_sum = total_el_core;
        ms->rms_res = rms_res; ms->rms_dphi = rms_dphi; ms->rms_dY = rms_dY;
        ms->energy_diff_rel = edr; ms->vol_err_rel = ver;
    }
    return PFGB_OK;
}

// ---------------------------------------------------------------------------
// construction
// ---------------------------------------------------------------------------
static void build_physc(pfgb_ctx *c) {
    const pfgb_params &P = c->p;
    PhysC &k = c->pc;
    memset(&k, 0, sizeof(k));
    k.dt = P.dt;
    k.invN = 1.0 / (double)c->g.N;
    k.W = P.W; k.kappa = P.kappa_phi; k.Lphi = P.L_phi;
    k.Da = P.D_alpha; k.Dc = P.D_compound;
    k.vA = P.v_A; k.vB = P.v_B; k.Vm0 = P.Vm_alpha_0; k.dVm = P.dVm_alpha_dxB; k.Vmc = P.Vm_compound;
    k.mu0 = P.mu0_compound; k.eiv = P.eps_iso_over_vB; k.Yclip = P.Y_clip; k.xBeps = P.xB_eps;
    k.hscale = P.Y_rhs_term_h_scale;
    for (int i = 0; i < 6; ++i) { k.e00[i] = P.eps00[i]; k.E0[i] = P.E0[i]; }
    for (int i = 0; i < 21; ++i) { k.S[i] = P.S[i]; k.Sp[i] = P.S_p[i]; }
    k.gp = P.model_mode == PFGB_MODEL_GP_ZONE;
    k.gp_el = k.gp && P.gp_elastic_enabled;
    k.act_eta = P.gp_elastic_active_eta;
    k.act_phi = P.gp_elastic_active_phi;
    k.elastic = P.elastic_enabled;
    // phi_elastic_coupling_enabled (main_cuda.cu:24868)
    k.coupling = P.elastic_enabled && (!k.gp_el || P.gp_elastic_active_phi);
    k.zm = P.zero_mode_enabled;
    // the q split evaluates mu and J at phi^{n+1} whatever the previous-level
    // switch says (phi_for_Y_explicit, main_cuda.cu:30286-30291); the switch
    // acts on nothing else there
    k.prev_level = P.enable_Y_rhs_previous_time_level && P.pf_y_update_mode != PFGB_Y_Q_TRANSPORT_SPLIT;
    k.disable_gamma = P.disable_Y_rhs_gamma_term;
    k.xb_raw = P.zero_mode_enabled;
    // gp_storage_coupling_enabled (main_cuda.cu:16767-16772)
    if (k.gp && (P.enable_legacy_gp_storage_coupling || !P.gp_barrier_only_mode))
        k.gpy = P.gp_y_update_mode == PFGB_GP_Y_OLD_RHS ? 1 : (P.gp_y_update_mode == PFGB_GP_Y_CONSERVATIVE_RHS ? 2 : 3);
    k.haeps = P.gp_h_alpha_eps;
    k.xbcap = 2.0;
    k.dx = P.dx; k.dy = P.dy; k.dz = P.dz;
    pfgb_thermo_const(P.temperature_K, P.mu_reference_scale, P.thermo_convex_extrapolation_enabled, &k.tc);
    k.shift = k.coupling ? P.elastic_shift_dimless : 0.0;
    k.Cdmu = P.mu0_compound - P.v_A * k.tc.GA_s - P.v_B * k.tc.GB_s - k.shift;
    k.dG = k.tc.GB_s - k.tc.GA_s;
    k.gpxB = P.gp_xB_fixed; k.gpW = P.gp_W_eta; k.gpkap = P.gp_kappa_eta; k.gpL = P.gp_L_eta;
    k.gpMGP = P.gp_M_GP; k.gpMb = P.gp_M_beta; k.gpeiso = P.gp_eps_iso; k.gpscale = P.gp_elastic_derivative_scale;
    {
        const double xg = clamp_eps(P.gp_xB_fixed, 1.0e-12);
        double oA, oB;
        thermo_mu_off<double>(k.tc, xg, oA, oB);
        k.gp_Cg = oA * (1.0 - xg) + oB * xg - P.gp_delta_g0;
    }
}

static pfgb_status dalloc(pfgb_ctx *c, void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        pfgb_set_error("cudaMalloc", e, __FILE__, __LINE__);
        return e == cudaErrorMemoryAllocation ? PFGB_ERR_NOMEM : PFGB_ERR_CUDA;
    }
    c->bytes += bytes;
    return PFGB_OK;
}

static pfgb_status upload_twiddles(pfgb_ctx *c, int axis, int n) {
    std::vector<double2> wd(n);
    std::vector<float2> wf(n);
    for (int m = 0; m < n; ++m) {
        // exact octant folding keeps the table symmetric to the last bit
        const double a = -2.0 * PFGB_PI * (double)m / (double)n;
        wd[m] = make_double2(cos(a), sin(a));
        wf[m] = make_float2((float)wd[m].x, (float)wd[m].y);
    }
    TRY(dalloc(c, &c->tw[0][axis], sizeof(double2) * n));
    TRY(dalloc(c, &c->tw[1][axis], sizeof(float2) * n));
    PFGB_CUDA_TRY(cudaMemcpy(c->tw[0][axis], wd.data(), sizeof(double2) * n, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->tw[1][axis], wf.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
    return PFGB_OK;
}

// B of the tensor-core 41-point stage (dft41_tc.cuh): B[n][j] for outputs
// k = n + 1 and pairing index j, as TF32 high parts (round to nearest, ties
// away, like cvt.rna) and the FP32 remainders, in the stage's shared-memory
// byte layout: hi matrix, then lo matrix
static uint32_t tf32_rna_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return (u + 0x1000u) & 0xFFFFE000u;
}
static pfgb_status upload_tc41_table(pfgb_ctx *c) {
    std::vector<unsigned char> tab(2 * tc41::B_BYTES, 0);
    for (int n = 0; n < tc41::NOUT; ++n)
        for (int j = 0; j < tc41::K; ++j) {
            const int k = n + 1;
            const double v = j < 20 ? cos(2.0 * PFGB_PI * (double)(((j + 1) * k) % 41) / 41.0)
                                    : sin(2.0 * PFGB_PI * (double)(((j - 19) * k) % 41) / 41.0);
            const uint32_t hb = tf32_rna_bits((float)v);
            float hi;
            memcpy(&hi, &hb, 4);
            const float lo = (float)(v - (double)hi);
            memcpy(&tab[tc41::b_offset(n, j)], &hi, 4);
            memcpy(&tab[tc41::B_BYTES + tc41::b_offset(n, j)], &lo, 4);
        }
    TRY(dalloc(c, &c->tc_btab, tab.size()));
    TRY(dalloc(c, (void **)&c->tc_err, sizeof(int)));
    PFGB_CUDA_TRY(cudaMemcpy(c->tc_btab, tab.data(), tab.size(), cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemset(c->tc_err, 0, sizeof(int)));
    return PFGB_OK;
}

static pfgb_status make_ktab(pfgb_ctx *c) {
    const pfgb_params &P = c->p;
    auto wrap = [](int i, int n, double d) {
        int ii = (i <= n / 2) ? i : i - n;
        return 2.0 * PFGB_PI * ii / (d * n);
    };
    auto cut = [](double k, double d) { return std::fabs(k) >= PFGB_PI * (2.0 / 3.0) / d; };
    std::vector<double> kx(P.Nx), ky(P.Ny), kz(c->g.NzC);
    std::vector<unsigned char> mx(P.Nx), my(P.Ny), mz(c->g.NzC);
    for (int i = 0; i < P.Nx; ++i) { kx[i] = wrap(i, P.Nx, P.dx); mx[i] = cut(kx[i], P.dx); }
    for (int j = 0; j < P.Ny; ++j) { ky[j] = wrap(j, P.Ny, P.dy); my[j] = cut(ky[j], P.dy); }
    for (int k = 0; k < c->g.NzC; ++k) { kz[k] = 2.0 * PFGB_PI * k / (P.dz * P.Nz); mz[k] = cut(kz[k], P.dz); }
    TRY(dalloc(c, (void **)&c->kx, sizeof(double) * P.Nx));
    TRY(dalloc(c, (void **)&c->ky, sizeof(double) * P.Ny));
    TRY(dalloc(c, (void **)&c->kz, sizeof(double) * c->g.NzC));
    TRY(dalloc(c, (void **)&c->mx, P.Nx));
    TRY(dalloc(c, (void **)&c->my, P.Ny));
    TRY(dalloc(c, (void **)&c->mz, c->g.NzC));
    PFGB_CUDA_TRY(cudaMemcpy(c->kx, kx.data(), sizeof(double) * P.Nx, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->ky, ky.data(), sizeof(double) * P.Ny, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->kz, kz.data(), sizeof(double) * c->g.NzC, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->mx, mx.data(), P.Nx, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->my, my.data(), P.Ny, cudaMemcpyHostToDevice));
    PFGB_CUDA_TRY(cudaMemcpy(c->mz, mz.data(), c->g.NzC, cudaMemcpyHostToDevice));
    return PFGB_OK;
}

// Spectral bounds of the increment operator L = -Gamma0 (h dC).  Gamma0 C0
// projects onto compatible strains and is self-adjoint in the C0 energy
// inner product, so L is too, and its Rayleigh quotient -<e, h dC e> /
// <e, C0 e> lies in [min(0, -mu_max), max(0, -mu_min)] for h in [0, 1],
// with mu the generalised eigenvalues of (dC, C0) (Voigt with engineering
// shear: the same quadratic forms as the stress kernels).  mu from the
// Cholesky factor C0 = L L^T and cyclic Jacobi on L^-1 dC L^-T.  The
// interval is widened by 2% of its length; false unless C0 is positive
// definite and the upper bound is below 1 (a convergent iteration).
static bool chebyshev_bounds(const double S[21], const double Sp[21], double *a, double *b) {
    static const int st[6] = {0, 6, 11, 15, 18, 20};
    auto V = [&](const double *c21, int i, int j) { if (i > j) std::swap(i, j); return c21[st[i] + j - i]; };
    double L[6][6] = {}, M[6][6], B[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j <= i; ++j) {
            double t = V(S, i, j);
            for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
            if (i == j) {
                if (!(t > 0.0)) return false;
                L[i][i] = std::sqrt(t);
            } else {
                L[i][j] = t / L[j][j];
            }
        }
    for (int col = 0; col < 6; ++col)       // M = L^-1 dC
        for (int i = 0; i < 6; ++i) {
            double t = V(Sp, i, col);
            for (int k = 0; k < i; ++k) t -= L[i][k] * M[k][col];
            M[i][col] = t / L[i][i];
        }
    for (int row = 0; row < 6; ++row)       // B = M L^-T: B^T = L^-1 M^T
        for (int i = 0; i < 6; ++i) {
            double t = M[row][i];
            for (int k = 0; k < i; ++k) t -= L[i][k] * B[row][k];
            B[row][i] = t / L[i][i];
        }
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) { tot += B[i][j] * B[i][j]; if (i != j) off += B[i][j] * B[i][j]; }
        if (!(off > 1e-30 * tot)) break;
        for (int p = 0; p < 5; ++p)
            for (int q = p + 1; q < 6; ++q) {
                if (std::fabs(B[p][q]) < 1e-300) continue;
                const double th = (B[q][q] - B[p][p]) / (2.0 * B[p][q]);
                const double t = (th >= 0.0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
                const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < 6; ++k) {
                    const double bp = B[k][p], bq = B[k][q];
                    B[k][p] = cs * bp - sn * bq;
                    B[k][q] = sn * bp + cs * bq;
                }
                for (int k = 0; k < 6; ++k) {
                    const double bp = B[p][k], bq = B[q][k];
                    B[p][k] = cs * bp - sn * bq;
                    B[q][k] = sn * bp + cs * bq;
                }
            }
    }
    double mn = B[0][0], mx = B[0][0];
    for (int i = 1; i < 6; ++i) { mn = std::min(mn, B[i][i]); mx = std::max(mx, B[i][i]); }
    double lo = std::min(0.0, -mx), hi = std::max(0.0, -mn);
    const double w = 0.02 * (hi - lo);
    lo -= w;
    hi += w;
    if (!std::isfinite(lo) || !std::isfinite(hi) || !(hi < 1.0)) return false;
    *a = lo;
    *b = hi;
    return true;
}

static pfgb_status validate(const pfgb_params *p) {
    if (p->Nx < 1 || p->Ny < 1 || p->Nz < 2 || p->Nx > PFGB_MAX_N || p->Ny > PFGB_MAX_N || p->Nz > PFGB_MAX_N) {
        pfgb_set_error_msg("grid %dx%dx%d outside [1..%d] (Nz >= 2)", p->Nx, p->Ny, p->Nz, PFGB_MAX_N);
        return PFGB_ERR_INVALID;
    }
    if (!(p->dx > 0 && p->dy > 0 && p->dz > 0 && p->dt > 0)) {
        pfgb_set_error_msg("dx, dy, dz, dt must be > 0");
        return PFGB_ERR_INVALID;
    }
    if (p->precision != PFGB_PREC_FP64 && p->precision != PFGB_PREC_FP32) {
        pfgb_set_error_msg("precision must be PFGB_PREC_FP64 or PFGB_PREC_FP32");
        return PFGB_ERR_INVALID;
    }
    if (p->elastic_precision != PFGB_PREC_FP32) {
        pfgb_set_error_msg("elastic_precision: only FP32 (the reference's elastic precision) is built");
        return PFGB_ERR_UNSUPPORTED;
    }
    if (p->mode != PFGB_MODE_DYNAMICS && p->mode != PFGB_MODE_MINIMIZE) {
        pfgb_set_error_msg("mode must be dynamics or minimize");
        return PFGB_ERR_INVALID;
    }
    if (p->mode == PFGB_MODE_MINIMIZE) {
        if ((p->model_mode != PFGB_MODEL_TWO_PHASE && !p->minimize_full_model) || p->zero_mode_enabled) {
            pfgb_set_error_msg("minimize is built for the full model (two_phase or gp_zone) and the phi-only "
                               "model (two_phase), with the zero mode off");
            return PFGB_ERR_UNSUPPORTED;
        }
        if (!(p->minimize_dt > 0)) {
            pfgb_set_error_msg("minimize_dt must be > 0");
            return PFGB_ERR_INVALID;
        }
    }
    if (p->model_mode != PFGB_MODEL_TWO_PHASE && p->model_mode != PFGB_MODEL_GP_ZONE) {
        pfgb_set_error_msg("model_mode must be two_phase or gp_zone");
        return PFGB_ERR_INVALID;
    }
    if (p->elastic_iter_max < 1 || p->elastic_iter_min < 0) {
        pfgb_set_error_msg("elastic_iter_max must be >= 1");
        return PFGB_ERR_INVALID;
    }
    if (p->elastic_chebyshev && p->elastic_enabled) {
        double a, b;
        if (!p->elastic_increment_form) {
            pfgb_set_error_msg("elastic_chebyshev needs elastic_increment_form = 1");
            return PFGB_ERR_INVALID;
        }
        if (!chebyshev_bounds(p->S, p->S_p, &a, &b)) {
            pfgb_set_error_msg("elastic_chebyshev: the elastic iteration's spectral bounds are not below 1 "
                               "(C0 not positive definite, or the stiffness contrast too large)");
            return PFGB_ERR_UNSUPPORTED;
        }
    }
    if (p->pf_y_update_mode < PFGB_Y_LAGGED_RHS || p->pf_y_update_mode > PFGB_Y_Q_TRANSPORT_SPLIT) {
        pfgb_set_error_msg("pf_y_update_mode: lagged_rhs, storage_exact, x_transport_projection_split or "
                           "q_transport_projection_split");
        return PFGB_ERR_UNSUPPORTED;
    }
    if (p->pf_y_update_mode == PFGB_Y_X_TRANSPORT_SPLIT &&
        (!(p->pf_matrix_storage_floor > 0.0 && p->pf_matrix_storage_floor <= 1.0) ||
         !(p->pf_composition_stabilizer_Dalpha_multiplier > 0.0) ||
         !std::isfinite(p->pf_composition_stabilizer_Dalpha_multiplier))) {
        // main_cuda.cu:1728-1739
        pfgb_set_error_msg("pf_matrix_storage_floor must be in (0,1] and "
                           "pf_composition_stabilizer_Dalpha_multiplier finite and > 0");
        return PFGB_ERR_INVALID;
    }
    if (p->gp_y_update_mode < PFGB_GP_Y_OLD_RHS || p->gp_y_update_mode > PFGB_GP_Y_CONSERVATIVE_RHS ||
        (p->gp_eta_mass_limiter != PFGB_GP_ETA_LIMITER_OFF &&
         p->gp_eta_mass_limiter != PFGB_GP_ETA_LIMITER_LOCAL_CLIP)) {
        // main_cuda.cu:1218-1225
        pfgb_set_error_msg("gp_y_update_mode: old_rhs, conservative_y_rhs, picard_storage or storage_exact; "
                           "gp_eta_mass_limiter: off or local_clip");
        return PFGB_ERR_INVALID;
    }
    if (p->model_mode == PFGB_MODEL_GP_ZONE && (p->enable_legacy_gp_storage_coupling || !p->gp_barrier_only_mode) &&
        p->mode != PFGB_MODE_DYNAMICS) {
        // gp_storage_coupling_enabled (main_cuda.cu:16767-16772): the
        // storage-coupled Y update is built for dynamics
        pfgb_set_error_msg("gp_zone minimize with the GP storage coupling (gp_barrier_only_mode=0 or "
                           "enable_legacy_gp_storage_coupling=1) is not built");
        return PFGB_ERR_UNSUPPORTED;
    }
    // the zero mode and minimize refuse every mode but lagged_rhs
    // (main_cuda.cu:24600-24612, 24692-24702); storage_exact and the x and q
    // splits without the GP storage coupling are the two_phase paths
    // (main_cuda.cu:27781-27783, 30564-30566, 30627-30628)
    if (p->pf_y_update_mode != PFGB_Y_LAGGED_RHS &&
        (p->zero_mode_enabled || p->model_mode != PFGB_MODEL_TWO_PHASE || p->mode != PFGB_MODE_DYNAMICS)) {
        pfgb_set_error_msg("pf_y_update_mode storage_exact / x_ or q_transport_projection_split: two_phase dynamics with "
                           "the zero mode off (the zero mode owns lagged_rhs; the GP storage-coupled modes are not "
                           "built)");
        return PFGB_ERR_UNSUPPORTED;
    }
    // PF-only conservative composition modes (main_cuda.cu:1697-1775, 24600-24612,
    // 24691-24702, 28487-28491)
    if (p->pf_composition_mode < PFGB_COMPOSITION_LEGACY || p->pf_composition_mode > PFGB_COMPOSITION_QALPHA ||
        p->pf_conservative_flux_strategy < PFGB_CONS_FLUX_PAIRWISE_LIMITED ||
        p->pf_conservative_flux_strategy > PFGB_CONS_FLUX_BACKWARD_EULER) {
        pfgb_set_error_msg("pf_composition_mode: legacy, ctot_conservative_split or "
                           "qalpha_conservative_local_transaction; pf_conservative_flux_strategy: pairwise_limited "
                           "or pairwise_backward_euler");
        return PFGB_ERR_INVALID;
    }
    if (p->pf_composition_mode != PFGB_COMPOSITION_LEGACY) {
        if (!(p->pf_conservative_bound_tol > 0.0) || !(p->pf_conservative_mass_tol > 0.0) ||
            !(p->pf_conservative_beta_support_eps > 0.0) || p->pf_conservative_max_subcycles < 1) {
            pfgb_set_error_msg("invalid PF conservative solver controls");
            return PFGB_ERR_INVALID;
        }
        if (p->model_mode != PFGB_MODEL_TWO_PHASE || p->zero_mode_enabled || p->mode != PFGB_MODE_DYNAMICS ||
            p->pf_y_update_mode != PFGB_Y_LAGGED_RHS) {
            pfgb_set_error_msg("conservative PF composition modes are PF-only two_phase dynamics with the zero mode "
                               "off and pf_y_update_mode lagged_rhs");
            return PFGB_ERR_UNSUPPORTED;
        }
        if ((p->Nx & 1) || (p->Ny & 1) || (p->Nz & 1)) {
            pfgb_set_error_msg("shared-face checkerboard solver requires even periodic dimensions");
            return PFGB_ERR_INVALID;
        }
    }
    if (p->elastic_warm_start_source < 0 || p->elastic_warm_start_source > 3) {
        pfgb_set_error_msg("elastic_warm_start_source must be 0, 1, 2 or 3");
        return PFGB_ERR_INVALID;
    }
    if (p->y_update_mass_projection_enabled &&
        (p->pf_composition_mode != PFGB_COMPOSITION_LEGACY || p->zero_mode_enabled)) {
        // main_cuda.cu:1719-1727 and 24691-24704
        pfgb_set_error_msg("y_update_mass_projection_enabled is refused with the conservative composition modes "
                           "and the zero mode");
        return PFGB_ERR_INVALID;
    }
    if (p->elastic_warm_start_extrapolate < 0 || p->elastic_warm_start_extrapolate > 5) {
        pfgb_set_error_msg("elastic_warm_start_extrapolate must be 0 (u^n) or the order 1 to 5");
        return PFGB_ERR_INVALID;
    }
    return PFGB_OK;
}

static void ctx_free(pfgb_ctx *c) {
    auto f = [](void *p) { if (p) cudaFree(p); };
    for (int a = 0; a < 2; ++a) for (int b = 0; b < 3; ++b) f(c->tw[a][b]);
    f(c->tc_btab);
    f(c->tc_err);
    f(c->kx); f(c->ky); f(c->kz); f(c->mx); f(c->my); f(c->mz);
    for (int i = 0; i < 2; ++i) f(c->phi[i]);
    f(c->eta[0]);
    if (c->eta[1] != c->eta[0]) f(c->eta[1]);
    f(c->Y); f(c->Yprev); f(c->dYdt);
    f(c->q); f(c->qb); f(c->divr);
    f(c->cstore); f(c->cmu);
    for (int i = 0; i < 4; ++i) f(c->S[i]);
    for (int i = 0; i < 6; ++i) { f(c->eps[i]); f(c->E[i]); }
    for (int i = 0; i < 3; ++i) f(c->U[i]);
    f(c->partials); f(c->dscal); f(c->stage);
    for (int i = 0; i < 6; ++i) f(c->sig[i]);
    for (int i = 0; i < 3; ++i) { f(c->Rk[i]); f(c->Dk[i]); f(c->Dkm[i]); for (int l = 0; l < 5; ++l) f(c->Uhist[l][i]); }
    f(c->mge); f(c->mlap);
    f(c->fno_in); f(c->fno_out);
    for (int i = 0; i < 3; ++i) f(c->Uhom[i]);
    for (auto e : c->pool) cudaEventDestroy(e);
    for (auto e : c->ev_rd) if (e) cudaEventDestroy(e);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->hscal) cudaFreeHost(c->hscal);
}

// float fields: Y = log x - log(1 - x) from the two float logarithms of the
// double x and 1 - x (each within an ulp of its value), so the FP64 pipe is
// not spent on a result stored in float; double fields keep logit_clip
template <typename T>
__device__ __forceinline__ T load_logit(double x, double eps, double Yclip) {
    if constexpr (sizeof(T) == 8) {
        return logit_clip(x, eps, Yclip);
    } else {
        const double xc = fmin(fmax(x, eps), 1.0 - eps);
        const float y = logf(float(xc)) - logf(float(1.0 - xc));
        return fminf(fmaxf(y, -float(Yclip)), float(Yclip));
    }
}

// MASS: also the block partials of the target mass of the zero mode
// (gpu_reduce_sum_xBtot, :28079-28086), taken on a first load only
template <typename T, bool MASS>
__global__ void k_load_state(const double *phi, const double *xB, const double *eta, const double *dYdt,
                             T *phi_o, T *eta_o, T *Y_o, T *dYdt_o, long long N, double xBeps, double Yclip,
                             double vB, double *partials) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const double p = phi[i], x = xB[i];
        phi_o[i] = (T)p;
        eta_o[i] = eta ? (T)eta[i] : T(0);
        dYdt_o[i] = dYdt ? (T)dYdt[i] : T(0);
        Y_o[i] = load_logit<T>(x, xBeps, Yclip);
        if (MASS) {
            const double h = pf_h(p);
            acc += (1.0 - h) * x + vB * h;
        }
    }
    if (MASS) {
        AccSum1 s{acc};
        block_reduce_acc(s);
        if (threadIdx.x == 0) reinterpret_cast<AccSum1 *>(partials)[blockIdx.x] = s;
    }
}

// FP32 fields hold the logit composition relative to its mean: Y* = Y - Yc
// with Yc = mean(Y) in FP64.  The Y update is linear in Y with the constant
// mode passed through unchanged, and every evaluation adds Yc back, so the
// shift changes no result in exact arithmetic; the float transforms of Y then
// carry roundoff in proportion to the spread of Y rather than to its mean
// (the logit of a dilute composition, about -3.5), and the stored Y* has the
// finer ulp of a centred value.  Y* is rounded once from the double logit
// (xB given) or the double Y (checkpoint restart).
template <typename T>
__global__ void k_sum_field(const T *f, long long N, double *partials) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x)
        acc += (double)f[i];
    AccSum1 s{acc};
    block_reduce_acc(s);
    if (threadIdx.x == 0) reinterpret_cast<AccSum1 *>(partials)[blockIdx.x] = s;
}

__global__ void k_center_logit(const double *xB, const double *Y, float *Y_o, long long N, double eps, double Yclip,
                               double shift) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const double y = Y ? Y[i] : logit_clip(xB[i], eps, Yclip);
        Y_o[i] = (float)(y - shift);
    }
}

// sets Yc to the mean of the loaded Y and stores Y - Yc (FP32 fields)
static pfgb_status center_logit(pfgb_ctx *c, const double *xB, const double *Y) {
    const int nb = 304;
    k_sum_field<float><<<nb, 256, 0, c->stream>>>((const float *)c->Y, c->g.N, c->partials);
    PFGB_CUDA_TRY(cudaGetLastError());
    TRY(reduce_to<AccSum1>(c, nb, DS_ZM));
    TRY(sync_read(c, DS_ZM, 1));
    const double m = c->hscal[DS_ZM] / (double)c->g.N;
    if (!std::isfinite(m)) {
        pfgb_set_error_msg("non-finite mean of the loaded logit composition");
        return PFGB_ERR_INVALID;
    }
    k_center_logit<<<nb, 256, 0, c->stream>>>(xB, Y, (float *)c->Y, c->g.N, c->p.xB_eps, c->p.Y_clip, m);
    PFGB_CUDA_TRY(cudaGetLastError());
    c->Yc = m;
    c->Yc_prev = m;
    return PFGB_OK;
}

template <typename T>
static pfgb_status load_device(pfgb_ctx *c, const double *phi, const double *xB, const double *eta,
                               const double *dYdt, bool keep_history) {
    const int nb = 304;
    const bool keep = keep_history && c->loaded;
    if (keep)
        k_load_state<T, false><<<nb, 256, 0, c->stream>>>(phi, xB, eta, dYdt, (T *)c->phi[c->cur],
                                                          (T *)c->eta[c->ecur], (T *)c->Y, (T *)c->dYdt, c->g.N,
                                                          c->p.xB_eps, c->p.Y_clip, c->p.v_B, c->partials);
    else
        k_load_state<T, true><<<nb, 256, 0, c->stream>>>(phi, xB, eta, dYdt, (T *)c->phi[c->cur],
                                                         (T *)c->eta[c->ecur], (T *)c->Y, (T *)c->dYdt, c->g.N,
                                                         c->p.xB_eps, c->p.Y_clip, c->p.v_B, c->partials);
    PFGB_CUDA_TRY(cudaGetLastError());
    c->Yc = 0.0;
    c->Yc_prev = 0.0;
    c->dYoff = 0.0;
    if (!keep) {
        TRY(reduce_to<AccSum1>(c, nb, DS_ZM));
        TRY(sync_read(c, DS_ZM, 1));
        c->target_mass = c->hscal[DS_ZM];
    }
    if constexpr (sizeof(T) == 4) TRY(center_logit(c, xB, nullptr));
    if (c->q) {   // q split: q = (1 - h) x of the loaded fields (main_cuda.cu:28051-28053)
        k_q_load<T><<<nb, 256, 0, c->stream>>>(phi, xB, (T *)c->q, c->g.N);
        PFGB_CUDA_TRY(cudaGetLastError());
    }
    if (c->cstore) {   // conservative modes: the storage of the loaded fields (main_cuda.cu:28054-28058)
        k_cons_load<<<nb, 256, 0, c->stream>>>(phi, xB, c->cstore, c->g.N,
                                               c->p.pf_composition_mode == PFGB_COMPOSITION_CTOT, c->p.v_B);
        PFGB_CUDA_TRY(cudaGetLastError());
        if (c->sig[0] && !keep)
            for (int i = 0; i < 6; ++i)
                PFGB_CUDA_TRY(cudaMemsetAsync(c->sig[i], 0, sizeof(float) * c->g.N, c->stream));
    }
    if (keep) return PFGB_OK;
    for (int i = 0; i < 6; ++i) PFGB_CUDA_TRY(cudaMemsetAsync(c->eps[i], 0, sizeof(float) * c->g.N, c->stream));
    c->warm_valid = 0;
    c->warm_count = 0;
    c->step = 0;
    c->zm_lambda = c->zm_residual = c->zm_derivative = 0.0;
    c->zm_iterations = c->zm_accepted = 0;
    c->min_iter = c->conv_count = c->converged_iter = c->xb_clamp = 0;
    c->lambda_vol = 0.0;
    c->prev_F_total = NAN;
    c->V0_target = c->p.minimize_V0;
    c->loaded = 1;
    return PFGB_OK;
}

static pfgb_status ensure_stage(pfgb_ctx *c) {
    if (c->stage) return PFGB_OK;
    return dalloc(c, (void **)&c->stage, sizeof(double) * 5 * (size_t)c->g.N);
}

static pfgb_status load_host(pfgb_ctx *c, const double *phi, const double *xB, const double *eta,
                             const double *dYdt, bool keep) {
    if (!c || !phi || !xB) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    TRY(ensure_stage(c));
    const size_t b = sizeof(double) * (size_t)c->g.N;
    double *dp = c->stage, *dx = c->stage + c->g.N;
    double *de = eta ? c->stage + 2 * c->g.N : nullptr, *dd = dYdt ? c->stage + 3 * c->g.N : nullptr;
    PFGB_CUDA_TRY(cudaMemcpyAsync(dp, phi, b, cudaMemcpyHostToDevice, c->stream));
    PFGB_CUDA_TRY(cudaMemcpyAsync(dx, xB, b, cudaMemcpyHostToDevice, c->stream));
    if (eta) PFGB_CUDA_TRY(cudaMemcpyAsync(de, eta, b, cudaMemcpyHostToDevice, c->stream));
    if (dYdt) PFGB_CUDA_TRY(cudaMemcpyAsync(dd, dYdt, b, cudaMemcpyHostToDevice, c->stream));
    return c->p.precision == PFGB_PREC_FP64 ? load_device<double>(c, dp, dx, de, dd, keep)
                                            : load_device<float>(c, dp, dx, de, dd, keep);
}

// checkpoint restart: phi, Y and dY/dt as stored (eta zero, as the
// reference restores it), and the mass ledger sum (1 - h) xB + v_B h of the
// stored phi and xB (gpu_reduce_sum_xBtot)
template <typename T>
__global__ void k_restore_state(const double *phi, const double *Y, const double *xB, const double *dYdt,
                                T *phi_o, T *eta_o, T *Y_o, T *dYdt_o, long long N, double vB, double *partials) {
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const double p = phi[i];
        phi_o[i] = (T)p;
        eta_o[i] = T(0);
        Y_o[i] = (T)Y[i];
        dYdt_o[i] = (T)dYdt[i];
        const double h = pf_h(p);
        acc += (1.0 - h) * xB[i] + vB * h;
    }
    AccSum1 s{acc};
    block_reduce_acc(s);
    if (threadIdx.x == 0) reinterpret_cast<AccSum1 *>(partials)[blockIdx.x] = s;
}

static pfgb_status checkpoint_context_ok(const pfgb_ctx *c, const char *what) {
    if (!c->p.zero_mode_enabled || c->p.model_mode != PFGB_MODEL_TWO_PHASE || c->p.mode != PFGB_MODE_DYNAMICS) {
        pfgb_set_error_msg("%s: checkpoints are the zero-mode dynamics contract (zero mode on, two_phase; the file "
                           "carries no eta)", what);
        return PFGB_ERR_UNSUPPORTED;
    }
    return PFGB_OK;
}

static bool accel_solver(const pfgb_params &P) {
    return P.elastic_enabled && (P.elastic_warm_start_enabled || P.elastic_residual_control_enabled);
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

pfgb_status pfgb_create(const pfgb_params *pin, int device, pfgb_ctx **out) {
    if (!pin || !out) return PFGB_ERR_INVALID;
    *out = nullptr;
    TRY(validate(pin));
    int ndev = 0;
    PFGB_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) {
        pfgb_set_error_msg("device %d not present (%d devices)", device, ndev);
        return PFGB_ERR_INVALID;
    }
    PFGB_CUDA_TRY(cudaSetDevice(device));
    pfgb_ctx *c = new pfgb_ctx();
    c->p = *pin;
    c->device = device;
    pfgb_params_finalize(&c->p);
    if (pin->mode == PFGB_MODE_MINIMIZE) c->p.dt = pin->minimize_dt;   // main_cuda.cu:24432-24435
    c->V0_target = pin->minimize_V0;
    c->g.Nx = pin->Nx; c->g.Ny = pin->Ny; c->g.Nz = pin->Nz; c->g.NzC = pin->Nz / 2 + 1;
    c->g.N = (long long)pin->Nx * pin->Ny * pin->Nz;
    c->g.Nk = (long long)pin->Nx * pin->Ny * c->g.NzC;
    pfgb_make_plan(pin->Nx, &c->plx);
    pfgb_make_plan(pin->Ny, &c->ply);
    pfgb_make_plan(pin->Nz, &c->plz);
    {
        // the strided-axis kernels copy column pairs with 16-byte accesses
        const bool e32 = pin->elastic_precision == PFGB_PREC_FP32, evenc = ((pin->Nz / 2 + 1) % 2) == 0;
        c->f246[0] = e32 && pin->Nx == f246::N && evenc;
        c->f246[1] = e32 && pin->Ny == f246::N && evenc;
        c->f246[2] = e32 && pin->Nz == f246::N;
    }
    build_physc(c);
    pfgb_status s = PFGB_OK;
    const size_t rs = pin->precision == PFGB_PREC_FP64 ? sizeof(double) : sizeof(float);
    const size_t N = (size_t)c->g.N, Nk = (size_t)c->g.Nk;
#define A_(ptr, b) if (s == PFGB_OK) s = dalloc(c, (void **)(ptr), (b))
    for (int i = 0; i < 2; ++i) { A_(&c->phi[i], rs * N); }
    if (c->pc.gp) { for (int i = 0; i < 2; ++i) { A_(&c->eta[i], rs * N); } }
    else { A_(&c->eta[0], rs * N); c->eta[1] = c->eta[0]; }
    A_(&c->Y, rs * N);
    A_(&c->Yprev, rs * N);
    A_(&c->dYdt, rs * N);
    if (pin->pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT) {
        A_(&c->q, rs * N);
        A_(&c->qb, rs * N);
        A_(&c->divr, rs * N);
    } else if (c->pc.gpy && pin->gp_eta_mass_limiter == PFGB_GP_ETA_LIMITER_LOCAL_CLIP) {
        A_(&c->divr, rs * N);   // the limiter's div J (second flux, right-hand side pass)
    }
    for (int i = 0; i < 4; ++i) { A_(&c->S[i], 2 * rs * Nk); }
    for (int i = 0; i < 6; ++i) { A_(&c->eps[i], sizeof(float) * N); }
    if (pin->elastic_enabled) {
        for (int i = 0; i < 6; ++i) { A_(&c->E[i], sizeof(float2) * Nk); }
        for (int i = 0; i < 3; ++i) { A_(&c->U[i], sizeof(float2) * Nk); }
        if (pin->elastic_increment_form &&
            (pin->elastic_warm_start_enabled || pin->elastic_residual_control_enabled)) {
            for (int i = 0; i < 3; ++i) { A_(&c->Rk[i], sizeof(float2) * Nk); A_(&c->Dk[i], sizeof(float2) * Nk); }
            double a = 0.0, b = 0.0;
            if (pin->elastic_chebyshev && chebyshev_bounds(pin->S, pin->S_p, &a, &b)) {   // checked in validate
                c->cheb_gam = 2.0 / (2.0 - a - b);
                c->cheb_sig = (b - a) / (2.0 - a - b);
                for (int i = 0; i < 3; ++i) A_(&c->Dkm[i], sizeof(float2) * Nk);
            }
        }
        if (pin->elastic_warm_start_extrapolate &&
            (pin->elastic_warm_start_enabled || pin->elastic_residual_control_enabled)) {
            for (int l = 0; l < pin->elastic_warm_start_extrapolate; ++l)
                for (int i = 0; i < 3; ++i) { A_(&c->Uhist[l][i], sizeof(float2) * Nk); }
        }
    }
    if (pin->pf_composition_mode != PFGB_COMPOSITION_LEGACY) {
        A_(&c->cstore, sizeof(double) * N);
        A_(&c->cmu, sizeof(double) * N);
    }
    // the stored stress: minimize, and the conservative modes, whose transport
    // runs before the step's elastic solve on the last solve's stress
    if (pin->mode == PFGB_MODE_MINIMIZE ||
        (pin->pf_composition_mode != PFGB_COMPOSITION_LEGACY && pin->elastic_enabled)) {
        for (int i = 0; i < 6; ++i) { A_(&c->sig[i], sizeof(float) * N); }
    }
    if (pin->mode == PFGB_MODE_MINIMIZE) {
        A_(&c->mge, rs * N);
        A_(&c->mlap, rs * N);
    }
    c->npartials = std::max<size_t>((size_t)pin->Nx * pin->Ny, 4096) * 8;
    A_(&c->partials, sizeof(double) * c->npartials);
    A_(&c->dscal, sizeof(double) * 64);
#undef A_
    if (s == PFGB_OK) s = make_ktab(c);
    if (s == PFGB_OK) s = upload_twiddles(c, 0, pin->Nx);
    if (s == PFGB_OK) s = upload_twiddles(c, 1, pin->Ny);
    if (s == PFGB_OK) s = upload_twiddles(c, 2, pin->Nz);
    if (s == PFGB_OK && pin->elastic_enabled) {
        c->tc_y = (pin->fft_tensor_cores & 1) && c->f246[1];
        c->tc_x = (pin->fft_tensor_cores & 2) && c->f246[0];
        c->tc_z = (pin->fft_tensor_cores & 4) && c->f246[2];
        if (c->tc_y || c->tc_x || c->tc_z) s = upload_tc41_table(c);
    }
    if (s == PFGB_OK) {
        cudaError_t e = cudaMallocHost((void **)&c->hscal, sizeof(double) * 64);
        if (e != cudaSuccess) { pfgb_set_error("cudaMallocHost", e, __FILE__, __LINE__); s = PFGB_ERR_CUDA; }
    }
    if (s == PFGB_OK && !c->pc.gp) {
        cudaError_t e = cudaMemset(c->eta[0], 0, rs * N);
        if (e != cudaSuccess) { pfgb_set_error("cudaMemset", e, __FILE__, __LINE__); s = PFGB_ERR_CUDA; }
    }
    // the table uploads and the memset above run on the legacy default
    // stream, which a non-blocking caller stream does not wait for
    if (s == PFGB_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { pfgb_set_error("cudaDeviceSynchronize", e, __FILE__, __LINE__); s = PFGB_ERR_CUDA; }
    }
    if (s != PFGB_OK) {
        ctx_free(c);
        delete c;
        return s;
    }
    *out = c;
    return PFGB_OK;
}

void pfgb_destroy(pfgb_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    ctx_free(c);
    delete c;
}

const char *pfgb_last_error(const pfgb_ctx *) { return pfgb_error_buffer(); }

pfgb_status pfgb_set_stream(pfgb_ctx *c, void *s) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));   // work queued on the previous stream
    c->stream = (cudaStream_t)s;
    return PFGB_OK;
}

size_t pfgb_device_bytes(const pfgb_ctx *c) { return c ? c->bytes : 0; }

pfgb_status pfgb_minimize(pfgb_ctx *c, int max_iter, int stop_on_convergence, pfgb_min_stats *st) {
    if (!c || max_iter < 0) return PFGB_ERR_INVALID;
    if (!c->loaded) { pfgb_set_error_msg("pfgb_minimize before pfgb_load_fields"); return PFGB_ERR_INVALID; }
    if (c->p.mode != PFGB_MODE_MINIMIZE) {
        pfgb_set_error_msg("pfgb_minimize needs a context created with mode=minimize");
        return PFGB_ERR_INVALID;
    }
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    if (st) memset(st, 0, sizeof(*st));
    for (int i = 0; i < max_iter; ++i) {
        pfgb_status s = c->p.precision == PFGB_PREC_FP64 ? minimize_once<double, float>(c, st)
                                                         : minimize_once<float, float>(c, st);
        if (s != PFGB_OK) return s;
        if (stop_on_convergence && c->converged_iter) break;
    }
    return PFGB_OK;
}

pfgb_status pfgb_sync(pfgb_ctx *c) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PFGB_OK;
}

pfgb_status pfgb_load_fields_device(pfgb_ctx *c, const double *phi, const double *xB, const double *eta,
                                    const double *dYdt) {
    if (!c || !phi || !xB) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    return c->p.precision == PFGB_PREC_FP64 ? load_device<double>(c, phi, xB, eta, dYdt, false)
                                            : load_device<float>(c, phi, xB, eta, dYdt, false);
}

pfgb_status pfgb_load_fields(pfgb_ctx *c, const double *phi, const double *xB, const double *eta,
                             const double *dYdt) {
    return load_host(c, phi, xB, eta, dYdt, false);
}

pfgb_status pfgb_set_fields(pfgb_ctx *c, const double *phi, const double *xB, const double *eta,
                            const double *dYdt) {
    return load_host(c, phi, xB, eta, dYdt, true);
}

pfgb_status pfgb_step(pfgb_ctx *c, int nsteps, pfgb_step_stats *st) {
    if (!c || nsteps < 0) return PFGB_ERR_INVALID;
    if (!c->loaded) { pfgb_set_error_msg("pfgb_step before pfgb_load_fields"); return PFGB_ERR_INVALID; }
    if (c->p.mode != PFGB_MODE_DYNAMICS) {
        pfgb_set_error_msg("pfgb_step drives mode=dynamics; this context is mode=minimize (pfgb_minimize)");
        return PFGB_ERR_INVALID;
    }
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    if (st) memset(st, 0, sizeof(*st));
    for (int i = 0; i < nsteps; ++i) {
        pfgb_status s = c->p.precision == PFGB_PREC_FP64 ? step_once<double, float>(c, st)
                                                         : step_once<float, float>(c, st);
        if (s != PFGB_OK) return s;
    }
    if (st) st->step = c->step;
    return PFGB_OK;
}

}  // extern "C"

template <typename T>
__global__ void k_export(const T *phi, const T *Y, const T *eta, const T *dYdt, long long N, double Yc,
                         double dYoff, int raw, double Yclip, double eps, double *ophi, double *oxB,
                         double *oY, double *oeta, double *odY) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const double y = double(Y[i]) + Yc;
        if (ophi) ophi[i] = double(phi[i]);
        if (oY) oY[i] = y;
        if (oxB) oxB[i] = raw ? sigmoid_raw(y) : sigmoid_clip(y, Yclip, eps);
        if (oeta) oeta[i] = double(eta[i]);
        if (odY) odY[i] = double(dYdt[i]) + dYoff;
    }
}

extern "C" {

pfgb_status pfgb_read_fields(pfgb_ctx *c, double *phi, double *xB, double *Y, double *eta, double *dYdt) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    const size_t b = sizeof(double) * (size_t)c->g.N;
    TRY(ensure_stage(c));
    if (!c->aux) PFGB_CUDA_TRY(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    for (auto &ev : c->ev_rd)
        if (!ev) PFGB_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    double *st = c->stage;
    const long long N = c->g.N;
    double *o[5] = {st, st + N, st + 2 * N, st + 3 * N, st + 4 * N};
    const int raw = c->p.zero_mode_enabled && c->step > 0;
    const bool fp64 = c->p.precision == PFGB_PREC_FP64;
    // the composition (an FP64 sigmoid per cell) on the side stream, after
    // the work queued so far; the other fields' export and copies meanwhile
    cudaError_t e = cudaSuccess;
    if (xB) {
        e = cudaEventRecord(c->ev_rd[0], c->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->aux, c->ev_rd[0], 0);
        if (e == cudaSuccess) {
            if (fp64)
                k_export<double><<<304, 256, 0, c->aux>>>(nullptr, (double *)c->Y, nullptr, nullptr, N, c->Yc,
                                                          c->dYoff, raw, c->p.Y_clip, c->p.xB_eps, nullptr, o[1],
                                                          nullptr, nullptr, nullptr);
            else
                k_export<float><<<304, 256, 0, c->aux>>>(nullptr, (float *)c->Y, nullptr, nullptr, N, c->Yc,
                                                         c->dYoff, raw, c->p.Y_clip, c->p.xB_eps, nullptr, o[1],
                                                         nullptr, nullptr, nullptr);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_rd[1], c->aux);
    }
    if (e == cudaSuccess) {
        if (fp64)
            k_export<double><<<304, 256, 0, c->stream>>>((double *)c->phi[c->cur], (double *)c->Y,
                                                         (double *)c->eta[c->ecur], (double *)c->dYdt, N, c->Yc,
                                                         c->dYoff, raw, c->p.Y_clip, c->p.xB_eps, o[0], nullptr,
                                                         o[2], o[3], o[4]);
        else
            k_export<float><<<304, 256, 0, c->stream>>>((float *)c->phi[c->cur], (float *)c->Y,
                                                        (float *)c->eta[c->ecur], (float *)c->dYdt, N, c->Yc,
                                                        c->dYoff, raw, c->p.Y_clip, c->p.xB_eps, o[0], nullptr,
                                                        o[2], o[3], o[4]);
        e = cudaGetLastError();
    }
    double *dst[5] = {phi, xB, Y, eta, dYdt};
    for (int i = 0; i < 5 && e == cudaSuccess; ++i)
        if (dst[i] && i != 1) e = cudaMemcpyAsync(dst[i], o[i], b, cudaMemcpyDeviceToHost, c->stream);
    if (xB && e == cudaSuccess) {
        e = cudaStreamWaitEvent(c->stream, c->ev_rd[1], 0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(xB, o[1], b, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) { pfgb_set_error("pfgb_read_fields", e, __FILE__, __LINE__); return PFGB_ERR_CUDA; }
    return PFGB_OK;
}

}  // extern "C"

template <typename T>
__global__ void k_stress_export(PhysCT<T> pc, ElasC<float> ec, const T *phi, const T *eta, const T *Y, double Yc,
                                float *const *eps, float *sig, long long N) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        float e[6], s[6];
        for (int a = 0; a < 6; ++a) e[a] = eps[a][i];
        const T xB = xB_of_Y<T>(pc, T(double(Y[i]) + Yc));
        stress_at<T, float>(pc, ec, phi[i], pc.gp ? eta[i] : T(0), xB, e, s);
        for (int a = 0; a < 6; ++a) sig[a * N + i] = s[a];
    }
}

extern "C" {

// sigma as the reference stores it after the elastic solve of the last step
// (phi, eta, xB of that step's start).
pfgb_status pfgb_read_elastic(pfgb_ctx *c, float *sigma6, float *strain6) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    const size_t N = (size_t)c->g.N;
    if (strain6)
        for (int a = 0; a < 6; ++a)
            PFGB_CUDA_TRY(cudaMemcpyAsync(strain6 + a * N, c->eps[a], sizeof(float) * N, cudaMemcpyDeviceToHost,
                                          c->stream));
    if (sigma6) {
        // the step swapped phi/eta buffers: the elastic solve saw the previous ones
        const int pc_ = c->step > 0 ? 1 - c->cur : c->cur;
        const int ec_ = (c->step > 0 && c->pc.gp) ? 1 - c->ecur : c->ecur;
        float *st = nullptr;
        pfgb_status s = dalloc(c, (void **)&st, sizeof(float) * 6 * N);
        if (s != PFGB_OK) return s;
        c->bytes -= sizeof(float) * 6 * N;
        float **dptrs = nullptr;
        PFGB_CUDA_TRY(cudaMalloc(&dptrs, sizeof(float *) * 6));
        PFGB_CUDA_TRY(cudaMemcpy(dptrs, c->eps, sizeof(float *) * 6, cudaMemcpyHostToDevice));
        const ElasC<float> ec = elas_consts<float>(c);
        // Y of the elastic solve: the copy the final Y pass kept, with the
        // offset of that step's start
        void *yv = c->step > 0 ? c->Yprev : c->Y;
        const double yc = c->step > 0 ? c->Yc_prev : c->Yc;
        if (c->p.precision == PFGB_PREC_FP64)
            k_stress_export<double><<<304, 256, 0, c->stream>>>(c->pc, ec, (double *)c->phi[pc_],
                                                                (double *)c->eta[ec_], (double *)yv, yc,
                                                                dptrs, st, (long long)N);
        else
            k_stress_export<float><<<304, 256, 0, c->stream>>>(phys_as<float>(c->pc), ec, (float *)c->phi[pc_],
                                                               (float *)c->eta[ec_], (float *)yv, yc, dptrs,
                                                               st, (long long)N);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(sigma6, st, sizeof(float) * 6 * N, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(st);
        cudaFree(dptrs);
        if (e != cudaSuccess) { pfgb_set_error("pfgb_read_elastic", e, __FILE__, __LINE__); return PFGB_ERR_CUDA; }
    }
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PFGB_OK;
}

}  // extern "C"

// training pair: cold solve with u_hom kept, then the model inputs and the
// real-space correction (U - U_hom) / N
template <typename T>
static pfgb_status training_pair(pfgb_ctx *c, float *in8, float *tgt3, pfgb_step_stats *st) {
    using T2e = float2;
    c->Yc_prev = c->Yc;
    c->pair_mode = 1;
    pfgb_status s = elastic_solve<T, float>(c, st);
    c->pair_mode = 0;
    TRY(s);
    T2e *E0 = (T2e *)c->E[0], *E1 = (T2e *)c->E[1], *E2 = (T2e *)c->E[2];
    {
        ProfScope ps(c, {"pair_difference", 9.0 * (double)c->g.Nk * sizeof(T2e)});
        k_sub3<float><<<1216, 256, 0, c->stream>>>(E0, E1, E2, (const T2e *)c->U[0], (const T2e *)c->U[1],
                                                   (const T2e *)c->U[2], (const T2e *)c->Uhom[0],
                                                   (const T2e *)c->Uhom[1], (const T2e *)c->Uhom[2], c->g.Nk);
        PFGB_CUDA_TRY(cudaGetLastError());
    }
    AxisIO<float, 3, 3> io;
    for (int i = 0; i < 3; ++i) { io.in[i] = (const T2e *)c->E[i]; io.out[i] = (T2e *)c->E[i]; }
    TRY((launch_axis<float, 3, 3, +1, 0>(c, 2, io, OpCopy<float, 3>{}, "x_inv3")));
    TRY((launch_axis<float, 3, 3, +1, 0>(c, 1, io, OpCopy<float, 3>{}, "y_inv3")));
    TRY((launch_z<float, 3, 0>(c, OpReal3Out<float>{E0, E1, E2, tgt3, c->g.N, c->g.NzC, (float)(1.0 / (double)c->g.N)},
                               "z_pair_c2r", 3.0 * (double)c->g.N * sizeof(float))));
    return launch_fno_inputs<T, float>(c, in8);
}

extern "C" {

pfgb_status pfgb_set_warm_start_model(pfgb_ctx *c, pfgb_fno *f) {
    if (!c) return PFGB_ERR_INVALID;
    if (!f) { c->fno = nullptr; return PFGB_OK; }
    pfgb_fno_config cfg;
    TRY(pfgb_fno_get_config(f, &cfg));
    if (cfg.Nx != c->g.Nx || cfg.Ny != c->g.Ny || cfg.Nz != c->g.Nz || pfgb_fno_device(f) != c->device) {
        pfgb_set_error_msg("warm-start model is on %dx%dx%d (device %d), the context on %dx%dx%d (device %d)", cfg.Nx,
                           cfg.Ny, cfg.Nz, pfgb_fno_device(f), c->g.Nx, c->g.Ny, c->g.Nz, c->device);
        return PFGB_ERR_INVALID;
    }
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    if (!c->fno_in) {
        PFGB_CUDA_TRY(cudaMalloc(&c->fno_in, sizeof(float) * 8 * (size_t)c->g.N));
        PFGB_CUDA_TRY(cudaMalloc(&c->fno_out, sizeof(float) * 3 * (size_t)c->g.N));
        c->bytes += sizeof(float) * 11 * (size_t)c->g.N;
    }
    c->fno = f;
    return PFGB_OK;
}

pfgb_status pfgb_elastic_training_pair(pfgb_ctx *c, float *d_in8, float *d_target3, pfgb_step_stats *st) {
    if (!c || !d_in8 || !d_target3) return PFGB_ERR_INVALID;
    const pfgb_params &P = c->p;
    if (!c->loaded) { pfgb_set_error_msg("training pair: no fields loaded"); return PFGB_ERR_INVALID; }
    if (!P.elastic_enabled || !P.elastic_warm_start_enabled || !P.elastic_residual_control_enabled) {
        pfgb_set_error_msg("training pair: needs elastic_enabled, elastic_warm_start_enabled and "
                           "elastic_residual_control_enabled");
        return PFGB_ERR_UNSUPPORTED;
    }
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    if (!c->Uhom[0]) {
        for (int i = 0; i < 3; ++i) PFGB_CUDA_TRY(cudaMalloc(&c->Uhom[i], sizeof(float2) * (size_t)c->g.Nk));
        c->bytes += 3 * sizeof(float2) * (size_t)c->g.Nk;
    }
    pfgb_step_stats local{};
    pfgb_step_stats *sp = st ? st : &local;
    sp->elastic_iterations_total = 0;
    return c->p.precision == PFGB_PREC_FP64 ? training_pair<double>(c, d_in8, d_target3, sp)
                                            : training_pair<float>(c, d_in8, d_target3, sp);
}

pfgb_status pfgb_init_fields(pfgb_ctx *c) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    TRY(ensure_stage(c));
    double *dp = c->stage, *dx = c->stage + c->g.N;
    TRY(pfgb_seed_fields_device(&c->p, dp, dx, c->partials, c->stream));
    return c->p.precision == PFGB_PREC_FP64 ? load_device<double>(c, dp, dx, nullptr, nullptr, false)
                                            : load_device<float>(c, dp, dx, nullptr, nullptr, false);
}

pfgb_status pfgb_checkpoint_save(pfgb_ctx *c, const char *path, const char *initial_state_class,
                                 const char *fixture_manifest_sha256,
                                 const char *profile_library_manifest_sha256) {
    if (!c || !path) return PFGB_ERR_INVALID;
    TRY(checkpoint_context_ok(c, "pfgb_checkpoint_save"));
    if (!c->loaded) { pfgb_set_error_msg("pfgb_checkpoint_save: no fields loaded"); return PFGB_ERR_INVALID; }
    const bool accel = accel_solver(c->p);
    if (accel && (!c->warm_valid || c->step < 1)) {
        pfgb_set_error_msg("pfgb_checkpoint_save: refusing to checkpoint an invalid elastic warm state at step %d",
                           c->step);
        return PFGB_ERR_INVALID;
    }
    pfgb_checkpoint_state st;
    std::memset(&st, 0, sizeof(st));
    TRY(pfgb_checkpoint_provenance_for(&c->p, initial_state_class, fixture_manifest_sha256,
                                       profile_library_manifest_sha256, &st.provenance));
    const size_t N = (size_t)c->g.N, Nk = (size_t)c->g.Nk;
    std::vector<double> phi(N), Y(N), xB(N), dYdt(N);
    std::vector<float> u;
    TRY(pfgb_read_fields(c, phi.data(), xB.data(), Y.data(), nullptr, dYdt.data()));
    if (accel) {
        u.resize(6 * Nk);
        TRY(pfgb_read_displacement_k(c, u.data()));
    }
    st.accepted_step = (uint64_t)c->step;
    st.nx = c->g.Nx; st.ny = c->g.Ny; st.nz = c->g.Nz;
    st.elastic_present = accel ? 1 : 0;
    st.dt_code = c->p.dt;
    st.temperature_K = c->p.temperature_C + 273.15;
    st.target_mass_code = c->target_mass;
    st.last_lambda = c->zm_lambda;
    st.last_residual_code = c->zm_residual;
    st.last_derivative_code = c->zm_derivative;
    st.last_iterations = c->zm_iterations;
    st.accepted_zero_mode_steps = c->zm_accepted;
    st.elastic_source_field_step = accel ? (uint64_t)(c->step - 1) : 0;
    st.elastic_last_iterations = accel ? c->el_iterations : 0;
    st.elastic_last_relative_residual = accel ? c->el_residual : 0.0;
    st.phi = phi.data(); st.Y = Y.data(); st.xB = xB.data(); st.dY_dt_prev = dYdt.data();
    st.displacement_k = accel ? u.data() : nullptr;
    return pfgb_checkpoint_write_file(path, &st);
}

pfgb_status pfgb_checkpoint_restore(pfgb_ctx *c, const char *path, const char *initial_state_class,
                                    const char *fixture_manifest_sha256,
                                    const char *profile_library_manifest_sha256) {
    if (!c || !path) return PFGB_ERR_INVALID;
    TRY(checkpoint_context_ok(c, "pfgb_checkpoint_restore"));
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    pfgb_checkpoint_provenance expect;
    TRY(pfgb_checkpoint_provenance_for(&c->p, initial_state_class, fixture_manifest_sha256,
                                       profile_library_manifest_sha256, &expect));
    const size_t N = (size_t)c->g.N, Nk = (size_t)c->g.Nk;
    std::vector<double> phi(N), Y(N), xB(N), dYdt(N);
    std::vector<float> u(6 * Nk);
    pfgb_checkpoint_state st;
    std::memset(&st, 0, sizeof(st));
    st.nx = c->g.Nx; st.ny = c->g.Ny; st.nz = c->g.Nz;
    st.phi = phi.data(); st.Y = Y.data(); st.xB = xB.data(); st.dY_dt_prev = dYdt.data();
    st.displacement_k = u.data();
    TRY(pfgb_checkpoint_read_file(path, &expect, &st));
    if (st.dt_code != c->p.dt || st.temperature_K != c->p.temperature_C + 273.15) {
        pfgb_set_error_msg("checkpoint %s: restart grid/dt/temperature mismatch", path);
        return PFGB_ERR_INVALID;
    }
    const bool accel = accel_solver(c->p);
    if (accel && !st.elastic_present) {
        pfgb_set_error_msg("checkpoint %s: accelerated elastic restart lacks the V4 warm state", path);
        return PFGB_ERR_INVALID;
    }
    TRY(ensure_stage(c));
    double *d = c->stage;
    const size_t b = sizeof(double) * N;
    PFGB_CUDA_TRY(cudaMemcpyAsync(d, phi.data(), b, cudaMemcpyHostToDevice, c->stream));
    PFGB_CUDA_TRY(cudaMemcpyAsync(d + N, Y.data(), b, cudaMemcpyHostToDevice, c->stream));
    PFGB_CUDA_TRY(cudaMemcpyAsync(d + 2 * N, xB.data(), b, cudaMemcpyHostToDevice, c->stream));
    PFGB_CUDA_TRY(cudaMemcpyAsync(d + 3 * N, dYdt.data(), b, cudaMemcpyHostToDevice, c->stream));
    const int nb = 304;
    if (c->p.precision == PFGB_PREC_FP64)
        k_restore_state<double><<<nb, 256, 0, c->stream>>>(d, d + N, d + 2 * N, d + 3 * N, (double *)c->phi[c->cur],
                                                           (double *)c->eta[c->ecur], (double *)c->Y,
                                                           (double *)c->dYdt, c->g.N, c->p.v_B, c->partials);
    else
        k_restore_state<float><<<nb, 256, 0, c->stream>>>(d, d + N, d + 2 * N, d + 3 * N, (float *)c->phi[c->cur],
                                                          (float *)c->eta[c->ecur], (float *)c->Y, (float *)c->dYdt,
                                                          c->g.N, c->p.v_B, c->partials);
    PFGB_CUDA_TRY(cudaGetLastError());
    TRY(reduce_to<AccSum1>(c, nb, DS_ZM));
    TRY(sync_read(c, DS_ZM, 1));
    const double mass = c->hscal[DS_ZM];
    if (!std::isfinite(mass) ||
        std::fabs(mass - st.target_mass_code) > 1.0e-12 * std::max(std::fabs(st.target_mass_code), 1.0)) {
        pfgb_set_error_msg("checkpoint %s: field ledger does not match the frozen zero-mode target: current=%.17e "
                           "target=%.17e", path, mass, st.target_mass_code);
        c->loaded = 0;
        return PFGB_ERR_ZERO_MODE;
    }
    if (accel) {
        for (int a = 0; a < 3; ++a)
            PFGB_CUDA_TRY(cudaMemcpyAsync(c->U[a], u.data() + 2 * a * Nk, sizeof(float2) * Nk,
                                          cudaMemcpyHostToDevice, c->stream));
    }
    for (int i = 0; i < 6; ++i) PFGB_CUDA_TRY(cudaMemsetAsync(c->eps[i], 0, sizeof(float) * N, c->stream));
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->Yc = 0.0;
    c->Yc_prev = 0.0;
    c->dYoff = 0.0;
    if (c->p.precision != PFGB_PREC_FP64) TRY(center_logit(c, nullptr, d + N));
    c->target_mass = st.target_mass_code;
    c->zm_lambda = st.last_lambda;
    c->zm_residual = st.last_residual_code;
    c->zm_derivative = st.last_derivative_code;
    c->zm_iterations = st.last_iterations;
    c->zm_accepted = st.accepted_zero_mode_steps;
    c->warm_valid = accel ? 1 : 0;
    c->warm_count = accel ? 1 : 0;
    c->el_iterations = st.elastic_last_iterations;
    c->el_residual = st.elastic_last_relative_residual;
    c->step = (int)st.accepted_step;
    c->min_iter = c->conv_count = c->converged_iter = c->xb_clamp = 0;
    c->loaded = 1;
    return PFGB_OK;
}

pfgb_status pfgb_read_displacement_k(pfgb_ctx *c, float *u3) {
    if (!c || !u3) return PFGB_ERR_INVALID;
    if (!c->p.elastic_enabled) return PFGB_ERR_UNSUPPORTED;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    const size_t Nk = (size_t)c->g.Nk;
    for (int a = 0; a < 3; ++a)
        PFGB_CUDA_TRY(cudaMemcpyAsync(u3 + 2 * a * Nk, c->U[a], sizeof(float2) * Nk, cudaMemcpyDeviceToHost,
                                      c->stream));
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return PFGB_OK;
}

}  // extern "C"

struct AccDiag {
    static constexpr bool kActive = true;
    double vf, mass, xb, nin, pmn, pmx, xmn, xmx, nif;
    __device__ static AccDiag identity() { return {0, 0, 0, 0, 1e300, -1e300, 1e300, -1e300, 0}; }
    __device__ static AccDiag combine(AccDiag a, const AccDiag &b) {
        a.vf += b.vf; a.mass += b.mass; a.xb += b.xb; a.nin += b.nin; a.nif += b.nif;
        a.pmn = fmin(a.pmn, b.pmn); a.pmx = fmax(a.pmx, b.pmx);
        a.xmn = fmin(a.xmn, b.xmn); a.xmx = fmax(a.xmx, b.xmx);
        return a;
    }
    __device__ static AccDiag shfl_down(AccDiag a, int o) {
        AccDiag r;
        double *pa = reinterpret_cast<double *>(&a), *pr = reinterpret_cast<double *>(&r);
#pragma unroll
        for (int i = 0; i < 9; ++i) pr[i] = __shfl_down_sync(0xffffffffu, pa[i], o);
        return r;
    }
};

template <typename T>
__global__ void k_diag(const T *phi, const T *Y, const T *eta, long long N, double Yc, int raw, double Yclip,
                       double eps, double vB, double xgp, AccDiag *part) {
    AccDiag a = AccDiag::identity();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N;
         i += (long long)gridDim.x * blockDim.x) {
        const double p = double(phi[i]);
        const double y = double(Y[i]) + Yc;
        const double x = raw ? sigmoid_raw(y) : sigmoid_clip(y, Yclip, eps);
        const double h = pf_h(p);
        a.vf += pf_h(clamp01(p));             // reduce_sum_h_kernel (:5580)
        if (eta) {                             // GP storage coupling: reduce_sum_xBtot_gp_kernel (:3830)
            const double he = pf_h(double(eta[i]));
            a.mass += (1.0 - h) * (1.0 - he) * x + (1.0 - h) * he * xgp + h;
        } else {
            a.mass += (1.0 - h) * x + vB * h;  // reduce_sum_xBtot_kernel (:3792)
        }
        a.xb += x;
        a.nin += p > 0.5 ? 1.0 : 0.0;                 // reduce_sum_N_in_N_if_kernel (:3746)
        a.nif += (p > 0.12 && p < 0.88) ? 1.0 : 0.0;
        a.pmn = fmin(a.pmn, p); a.pmx = fmax(a.pmx, p);
        a.xmn = fmin(a.xmn, x); a.xmx = fmax(a.xmx, x);
    }
    block_reduce_acc(a);
    if (threadIdx.x == 0) part[blockIdx.x] = a;
}

extern "C" {

pfgb_status pfgb_diagnostics(pfgb_ctx *c, pfgb_diag *out) {
    if (!c || !out) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaSetDevice(c->device));
    const int nb = 304;
    const int raw = c->p.zero_mode_enabled && c->step > 0;
    // the model's xBtot (gpu_reduce_sum_model_xBtot, main_cuda.cu:21215-21224)
    void *eta = c->pc.gpy ? c->eta[c->ecur] : nullptr;
    if (c->p.precision == PFGB_PREC_FP64)
        k_diag<double><<<nb, 256, 0, c->stream>>>((double *)c->phi[c->cur], (double *)c->Y, (const double *)eta,
                                                  c->g.N, c->Yc, raw, c->p.Y_clip, c->p.xB_eps, c->p.v_B,
                                                  c->p.gp_xB_fixed, (AccDiag *)c->partials);
    else
        k_diag<float><<<nb, 256, 0, c->stream>>>((float *)c->phi[c->cur], (float *)c->Y, (const float *)eta,
                                                 c->g.N, c->Yc, raw, c->p.Y_clip, c->p.xB_eps, c->p.v_B,
                                                 c->p.gp_xB_fixed, (AccDiag *)c->partials);
    PFGB_CUDA_TRY(cudaGetLastError());
    TRY(reduce_to<AccDiag>(c, nb, 24));
    TRY(sync_read(c, 24, 9));
    const double *h = c->hscal + 24;
    const double N = (double)c->g.N;
    out->vf_precip = h[0] / N;
    out->mass_xBtot = h[1];
    out->mean_xB = h[2] / N;
    out->n_in = h[3];
    out->phi_min = h[4]; out->phi_max = h[5];
    out->xB_min = h[6]; out->xB_max = h[7];
    out->n_if = h[8];
    return PFGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// standalone 3D transforms (test / tooling entry points)
// ---------------------------------------------------------------------------
template <typename T>
struct OpRealIn {
    using Acc = NoAcc;
    const T *src; cplx_t<T> *dst; int NzC;
    __device__ void point(long long cell, const T *, T *out, Acc &) const { out[0] = src[cell]; }
    __device__ void load_spec(long long, int, cplx_t<T> *) const {}
    __device__ void store_spec(long long row, int k, const cplx_t<T> *v) const { dst[row * NzC + k] = v[0]; }
};
template <typename T>
struct OpRealOut {
    using Acc = NoAcc;
    const cplx_t<T> *src; T *dst; int NzC;
    __device__ void load_spec(long long row, int k, cplx_t<T> *v) const { v[0] = src[row * NzC + k]; }
    __device__ void point(long long cell, const T *in, T *, Acc &) const { dst[cell] = in[0]; }
    __device__ void store_spec(long long, int, const cplx_t<T> *) const {}
};

static pfgb_status fft_ctx_init(pfgb_ctx *c, int Nx, int Ny, int Nz, void *stream) {
    if (Nx < 1 || Ny < 1 || Nz < 2 || Nx > PFGB_MAX_N || Ny > PFGB_MAX_N || Nz > PFGB_MAX_N) {
        pfgb_set_error_msg("transform size %dx%dx%d outside [1..%d] (Nz >= 2)", Nx, Ny, Nz, PFGB_MAX_N);
        return PFGB_ERR_INVALID;
    }
    c->stream = (cudaStream_t)stream;
    c->g.Nx = Nx; c->g.Ny = Ny; c->g.Nz = Nz; c->g.NzC = Nz / 2 + 1;
    c->g.N = (long long)Nx * Ny * Nz;
    c->g.Nk = (long long)Nx * Ny * c->g.NzC;
    pfgb_make_plan(Nx, &c->plx);
    pfgb_make_plan(Ny, &c->ply);
    pfgb_make_plan(Nz, &c->plz);
    TRY(upload_twiddles(c, 0, Nx));
    TRY(upload_twiddles(c, 1, Ny));
    TRY(upload_twiddles(c, 2, Nz));
    return PFGB_OK;
}

static void fft_ctx_free(pfgb_ctx *c) {
    cudaStreamSynchronize(c->stream);
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 3; ++b)
            if (c->tw[a][b]) cudaFree(c->tw[a][b]);
}

template <typename T>
static pfgb_status fft_r2c_impl(pfgb_ctx *c, const T *in, cplx_t<T> *out) {
    TRY((launch_z<T, 0, 1>(c, OpRealIn<T>{in, out, c->g.NzC}, "z_r2c", (double)c->g.N * sizeof(T))));
    AxisIO<T, 1, 1> io;
    io.in[0] = out; io.out[0] = out;
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 1, io, OpCopy<T, 1>{}, "y_fwd1")));
    TRY((launch_axis<T, 1, 1, -1, 0>(c, 2, io, OpCopy<T, 1>{}, "x_fwd1")));
    return PFGB_OK;
}
template <typename T>
static pfgb_status fft_c2r_impl(pfgb_ctx *c, cplx_t<T> *in, T *out) {
    AxisIO<T, 1, 1> io;
    io.in[0] = in; io.out[0] = in;
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 2, io, OpCopy<T, 1>{}, "x_inv1")));
    TRY((launch_axis<T, 1, 1, +1, 0>(c, 1, io, OpCopy<T, 1>{}, "y_inv1")));
    TRY((launch_z<T, 1, 0>(c, OpRealOut<T>{in, out, c->g.NzC}, "z_c2r", (double)c->g.N * sizeof(T))));
    return PFGB_OK;
}

// The line engines stage tiles with 16-byte cp.async copies from the
// buffers' base addresses, so caller buffers must be 16-byte aligned (every
// cudaMalloc'd pointer is).  Checked on the host before anything launches.
static pfgb_status check_transform_buffers(const void *in, const void *out) {
    if (!in || !out) {
        pfgb_set_error_msg("null device buffer");
        return PFGB_ERR_INVALID;
    }
    if ((((uintptr_t)in) | ((uintptr_t)out)) & 15u) {
        pfgb_set_error_msg("transform buffers must be 16-byte aligned (in %p, out %p)", in, out);
        return PFGB_ERR_INVALID;
    }
    return PFGB_OK;
}

extern "C" {

// the elastic iteration's y transform of six half spectra on the 246-point
// engine (test / tooling entry point)
void pfgb_set_tune_copies(int copies) { g_tune_copies.store(copies < 1 ? 1 : (copies > 16 ? 16 : copies)); }

size_t pfgb_tile_report(char *buf, size_t len) {
    std::string out;
    {
        std::lock_guard<std::mutex> lk(g_tile_mu);
        for (const auto &kv : g_tiles) {
            const TileRec &r = kv.second;
            char line[256];
            snprintf(line, sizeof(line), "%s n=%lld extents=%lld,%lld tile=%d %.4f ms rule=%d %.4f ms\n",
                     r.tag.c_str(), r.a, r.b, r.c, r.tile, (double)r.t_ms, r.rule, (double)r.t_rule_ms);
            out += line;
        }
    }
    if (buf && len) {
        const size_t m = std::min(len - 1, out.size());
        memcpy(buf, out.data(), m);
        buf[m] = '\0';
    }
    return out.size();
}

pfgb_status pfgb_fft_y246x6(int tensor_cores, int dir, int Nx, int NzC, void *spec6, void *stream) {
    if (!spec6 || (dir != -1 && dir != 1) || Nx < 1 || NzC < 2 || (NzC % 2) != 0 || NzC > PFGB_MAX_N) {
        pfgb_set_error_msg("pfgb_fft_y246x6: dir must be -1 or +1, Nx >= 1 and NzC even in [2, %d]", PFGB_MAX_N);
        return PFGB_ERR_INVALID;
    }
    TRY(check_transform_buffers(spec6, spec6));
    pfgb_ctx c;
    pfgb_status s = fft_ctx_init(&c, Nx, f246::N, 2 * (NzC - 1), stream);
    c.g.NzC = NzC;
    c.g.Nk = (long long)Nx * f246::N * NzC;
    const size_t per = sizeof(float2) * (size_t)c.g.Nk;
    for (int i = 0; i < 6; ++i) c.E[i] = (unsigned char *)spec6 + i * per;
    if (s == PFGB_OK && tensor_cores) {
        s = upload_tc41_table(&c);
        c.tc_y = true;
    }
    if (s == PFGB_OK) s = dir < 0 ? launch_y246<-1>(&c, "y_fwd6") : launch_y246<+1>(&c, "y_inv6");
    if (s == PFGB_OK && c.tc_err) {
        int te = 0;
        if (cudaMemcpyAsync(&te, c.tc_err, sizeof(int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
            cudaStreamSynchronize(c.stream) != cudaSuccess) s = PFGB_ERR_CUDA;
        else if (te) { pfgb_set_error_msg("tensor-core 41-point stage: a wait ran out"); s = PFGB_ERR_TIMEOUT; }
    }
    fft_ctx_free(&c);
    if (c.tc_btab) cudaFree(c.tc_btab);
    if (c.tc_err) cudaFree(c.tc_err);
    return s;
}

pfgb_status pfgb_fft3d_r2c(int precision, int Nx, int Ny, int Nz, const void *in, void *out, void *stream) {
    TRY(check_transform_buffers(in, out));
    pfgb_ctx c;
    pfgb_status s = fft_ctx_init(&c, Nx, Ny, Nz, stream);
    if (s == PFGB_OK)
        s = precision == PFGB_PREC_FP64 ? fft_r2c_impl<double>(&c, (const double *)in, (double2 *)out)
                                        : fft_r2c_impl<float>(&c, (const float *)in, (float2 *)out);
    fft_ctx_free(&c);
    return s;
}

// The half-spectrum input is used as workspace and is overwritten.
pfgb_status pfgb_fft3d_c2r(int precision, int Nx, int Ny, int Nz, const void *in, void *out, void *stream) {
    TRY(check_transform_buffers(in, out));
    pfgb_ctx c;
    pfgb_status s = fft_ctx_init(&c, Nx, Ny, Nz, stream);
    if (s == PFGB_OK)
        s = precision == PFGB_PREC_FP64 ? fft_c2r_impl<double>(&c, (double2 *)in, (double *)out)
                                        : fft_c2r_impl<float>(&c, (float2 *)in, (float *)out);
    fft_ctx_free(&c);
    return s;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// allocation-free forward transform: twiddle tables in a static device array
// ---------------------------------------------------------------------------
// Three tables (x, y, z), each starting on a 256-byte boundary.  Every call
// rewrites the tables it reads, on its own stream, so no part of the array
// has to start at zero.  Calls overlapping on one device race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[PFGB_NOALLOC_SCRATCH_BYTES];

static constexpr int kNoallocMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_addr[kNoallocMaxDevices];

static size_t round256(size_t b) { return (b + 255) & ~(size_t)255; }

// w_a[m] = exp(-2 pi i m / n_a), the same table the allocating path uploads
template <typename T>
__global__ void k_fill_twiddles(unsigned char *base, int n0, int n1, int n2, size_t off1, size_t off2) {
    const int a = blockIdx.y;
    const int n = a == 0 ? n0 : (a == 1 ? n1 : n2);
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    cplx_t<T> *w = (cplx_t<T> *)(base + (a == 0 ? 0 : (a == 1 ? off1 : off2)));
    double s, co;
    sincospi(-2.0 * (double)m / (double)n, &s, &co);
    w[m].x = (T)co;
    w[m].y = (T)s;
}

// Address of the scratch array on the calling thread's current device,
// looked up once per device.
static pfgb_status noalloc_scratch(unsigned char **out) {
    int dev = -1;
    PFGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoallocMaxDevices) {
        pfgb_set_error_msg("device ordinal %d beyond the %d supported by the static scratch table", dev,
                           kNoallocMaxDevices);
        return PFGB_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
        void *p = nullptr;
        PFGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[dev] = p;
    }
    *out = (unsigned char *)g_noalloc_addr[dev];
    return PFGB_OK;
}

template <typename T>
static pfgb_status fft_r2c_noalloc(int Nx, int Ny, int Nz, const T *in, cplx_t<T> *out, void *stream) {
    const size_t off1 = round256(sizeof(cplx_t<T>) * (size_t)Nx);
    const size_t off2 = off1 + round256(sizeof(cplx_t<T>) * (size_t)Ny);
    const size_t need = off2 + round256(sizeof(cplx_t<T>) * (size_t)Nz);
    if (need > PFGB_NOALLOC_SCRATCH_BYTES) {
        pfgb_set_error_msg("%s transform %dx%dx%d needs %zu bytes of twiddle scratch; the static array holds %d",
                           sizeof(T) == 8 ? "FP64" : "FP32", Nx, Ny, Nz, need, PFGB_NOALLOC_SCRATCH_BYTES);
        return PFGB_ERR_INVALID;
    }
    unsigned char *base = nullptr;
    TRY(noalloc_scratch(&base));
    pfgb_ctx c;
    c.stream = (cudaStream_t)stream;
    c.g.Nx = Nx; c.g.Ny = Ny; c.g.Nz = Nz; c.g.NzC = Nz / 2 + 1;
    c.g.N = (long long)Nx * Ny * Nz;
    c.g.Nk = (long long)Nx * Ny * c.g.NzC;
    pfgb_make_plan(Nx, &c.plx);
    pfgb_make_plan(Ny, &c.ply);
    pfgb_make_plan(Nz, &c.plz);
    const int pi = sizeof(T) == 8 ? 0 : 1;
    c.tw[pi][0] = base;
    c.tw[pi][1] = base + off1;
    c.tw[pi][2] = base + off2;
    const int nmax = std::max(Nx, std::max(Ny, Nz));
    k_fill_twiddles<T><<<dim3((nmax + 255) / 256, 3), 256, 0, c.stream>>>(base, Nx, Ny, Nz, off1, off2);
    PFGB_CUDA_TRY(cudaGetLastError());
    pfgb_status s = fft_r2c_impl<T>(&c, in, out);
    c.tw[pi][0] = c.tw[pi][1] = c.tw[pi][2] = nullptr;
    return s;
}

extern "C" {

pfgb_status pfgb_fft3d_r2c_noalloc(int precision, int Nx, int Ny, int Nz, const void *in, void *out, void *stream) {
    TRY(check_transform_buffers(in, out));
    if (precision != PFGB_PREC_FP64 && precision != PFGB_PREC_FP32) {
        pfgb_set_error_msg("precision %d is neither PFGB_PREC_FP64 nor PFGB_PREC_FP32", precision);
        return PFGB_ERR_INVALID;
    }
    if (Nx < 1 || Ny < 1 || Nz < 2 || Nx > PFGB_MAX_N || Ny > PFGB_MAX_N || Nz > PFGB_MAX_N) {
        pfgb_set_error_msg("transform size %dx%dx%d outside [1..%d] (Nz >= 2)", Nx, Ny, Nz, PFGB_MAX_N);
        return PFGB_ERR_INVALID;
    }
    return precision == PFGB_PREC_FP64
               ? fft_r2c_noalloc<double>(Nx, Ny, Nz, (const double *)in, (double2 *)out, stream)
               : fft_r2c_noalloc<float>(Nx, Ny, Nz, (const float *)in, (float2 *)out, stream);
}

}  // extern "C"

extern "C" {

pfgb_status pfgb_profile_enable(pfgb_ctx *c, int on) {
    if (!c) return PFGB_ERR_INVALID;
    PFGB_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->prof = on ? 1 : 0;
    c->recs.clear();
    c->pool_used = 0;
    c->launches = 0;
    return PFGB_OK;
}

long long pfgb_profile_launches(const pfgb_ctx *c) { return c ? c->launches : -1; }

// Aggregate the recorded launches by tag.  Call with names == NULL to get
// the number of distinct tags; otherwise fills up to `cap` rows.
int pfgb_profile_read(pfgb_ctx *c, const char **names, double *ms, double *bytes, int *count, int cap) {
    if (!c) return -1;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return -1;
    std::vector<const char *> tags;
    std::vector<double> t, b;
    std::vector<int> n;
    for (auto &r : c->recs) {
        float e = 0.f;
        cudaEventElapsedTime(&e, r.a, r.b);
        size_t i = 0;
        while (i < tags.size() && strcmp(tags[i], r.tag) != 0) ++i;
        if (i == tags.size()) { tags.push_back(r.tag); t.push_back(0); b.push_back(0); n.push_back(0); }
        t[i] += e; b[i] += r.bytes; n[i] += 1;
    }
    if (names) {
        for (int i = 0; i < (int)tags.size() && i < cap; ++i) {
            names[i] = tags[i]; ms[i] = t[i]; bytes[i] = b[i]; count[i] = n[i];
        }
    }
    return (int)tags.size();
}

}  // extern "C"

// dft41_tc.cuh — the 41-point stage of the 246 = 6 x 41 line engine as a
// split-precision TF32 contraction on the fifth-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory).
//
// For one 41-point DFT with inputs y_0..y_40 and the symmetric pairing
// a_n = y_n + y_(41-n), b_n = y_n - y_(41-n) (n = 1..20):
//   X_k = y_0 + sum_n a_n cos(2 pi n k / 41) + DIR i sum_n b_n sin(2 pi n k / 41),
// valid for every k = 0..40.  With c = cos, s = sin:
//   Re X_k - Re y_0 = sum_n a_n.x c_nk + sum_n (-DIR b_n.y) s_nk
//   Im X_k - Im y_0 = sum_n a_n.y c_nk + sum_n ( DIR b_n.x) s_nk
// so each DFT is two rows of a real GEMM D = A B^T with K = 40:
//   A_re = [a.x (20) | -DIR b.y (20)], A_im = [a.y (20) | DIR b.x (20)],
//   B[n_out][j] = cos(2 pi (j+1) k / 41) (j < 20), sin(2 pi (j-19) k / 41)
//   (j >= 20), with k = n_out + 1 = 1..40; X_0 = y_0 + sum a stays on the
//   CUDA cores.
// Split precision (three terms): A = Ah + Al, B = Bh + Bl with the high parts
// rounded to TF32 (cvt.rna), and D = Ah Bh + Ah Bl + Al Bh accumulated in
// FP32 by the tensor core: about 22 significant bits, the FP32 engine's
// accuracy.  The sign of the sine part follows DIR through A, so one B
// serves both directions.
//
// Placement: one instance per thread; thread t of warp w owns TMEM lane
// 32 (w % 4) + (t % 32) of tile w / 4.  A tile is 128 instances (M = 128);
// a block's tiles run one after another through one 256-column TMEM
// allocation:
//   [0, 40) A_re hi  [40, 80) A_re lo  [80, 120) A_im hi  [120, 160) A_im lo
//   [160, 208) D_re   [208, 256) D_im    (N = 48; columns 40..47 unused)
// The A rows are written from registers with tcgen05.st (no shared-memory
// staging); B (hi and lo, 6,400 bytes each) sits in shared memory in the
// canonical K-major layout without swizzle: core matrices of 8 outputs x 4
// k (128 bytes), 128 bytes between output groups, 640 bytes between k
// groups.  Only output groups 0..4 are stored: the MMA's sixth group (its
// unused columns 40..47) reads the next 128 bytes, which lie inside the
// shared allocation and only feed those unused columns.
#pragma once

#include <cstdint>

#include "fft246.cuh"

namespace tc41 {

constexpr int K = 40;
constexpr int NOUT = 40;
constexpr int NMMA = 48;
constexpr int NG = 5;                          // stored output groups of 8
constexpr int KG = K / 4;                      // k groups of 4
constexpr int B_BYTES = KG * NG * 128;         // one matrix (hi or lo): 6,400
constexpr int KSTEP_BYTES = 2 * NG * 128;      // one MMA consumes K = 8 = two k groups
constexpr int TMEM_COLS = 256;
constexpr int COL_ARE_HI = 0, COL_ARE_LO = 40, COL_AIM_HI = 80, COL_AIM_LO = 120, COL_DRE = 160, COL_DIM = 208;
// bounded wait on the MMA completion barrier (try_wait polls): far above
// the few thousand cycles a tile takes; on expiry the block records an
// error and leaves its outputs unwritten
constexpr int WAIT_POLLS = 1 << 22;

// byte offset of B[n][j] (n = output 0..39, j = 0..39) in one matrix
__host__ __device__ constexpr int b_offset(int n, int j) {
    return (j >> 2) * (NG * 128) + (n >> 3) * 128 + (n & 7) * 16 + (j & 3) * 4;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor, no swizzle (start, leading / stride byte
// offsets >> 4, descriptor version 1 of this architecture family)
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor: kind::tf32, D in FP32, A and B TF32 K-major, M x N
__device__ __forceinline__ constexpr uint32_t idesc(int m, int n) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, int ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, int ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void st8(uint32_t taddr, const float *v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr),
                 "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
                 "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
                 "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7]))
                 : "memory");
}
__device__ __forceinline__ void ld8(uint32_t taddr, float *v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr)
                 : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t d, uint32_t a, uint64_t b, uint32_t id, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d),
        "r"(a), "l"(b), "r"(id), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}
__device__ __forceinline__ void mbar_init(uint64_t *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the phase `parity` of the barrier to complete
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity) {
    uint32_t ok = 0;
    for (int it = 0; it < WAIT_POLLS && !ok; ++it) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
    }
    return ok != 0;
}

// block-level state of the tensor-core stage
struct Ctx {
    uint32_t tmem;        // base of the block's 256 columns
    uint64_t *mbar;       // MMA completion barrier
    uint32_t phase;       // parity of the next completion
    uint32_t b_hi, b_lo;  // shared addresses of B (hi, lo)
    int *err;             // set to 1 when a wait ran out
};

// the 30 MMAs of one tile (thread 0 of the block issues them)
__device__ __forceinline__ void issue_tile(const Ctx &c) {
    constexpr uint32_t id = idesc(128, NMMA);
    // the k-group stride is the leading byte offset, the output-group stride
    // the stride byte offset, for the K-major operand without swizzle
    constexpr uint32_t lbo = NG * 128, sbo = 128;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
        const uint32_t d = c.tmem + (part ? COL_DIM : COL_DRE);
        const uint32_t ah = c.tmem + (part ? COL_AIM_HI : COL_ARE_HI);
        const uint32_t al = c.tmem + (part ? COL_AIM_LO : COL_ARE_LO);
#pragma unroll
        for (int s = 0; s < K / 8; ++s) {
            const uint64_t bh = sdesc(c.b_hi + s * KSTEP_BYTES, lbo, sbo);
            const uint64_t bl = sdesc(c.b_lo + s * KSTEP_BYTES, lbo, sbo);
            mma(d, ah + 8 * s, bh, id, s > 0 ? 1u : 0u);
            mma(d, ah + 8 * s, bl, id, 1u);
            mma(d, al + 8 * s, bh, id, 1u);
        }
    }
    commit(c.mbar);
}

// Stage C of the 6 x 41 engine on the tensor cores, for either layout of
// f246::stage_c (element (line l, position p) at buf[p * PS + l * LS]):
// the block's NL * 6 items read their 41 inputs, the block synchronises,
// the outputs are written to positions k1 + 6 k.  All threads of the block
// call it.
template <int DIR, int PS, int LS>
__device__ __forceinline__ void stage_c(float2 *buf, Ctx &c) {
    using namespace f246;
    const int it = threadIdx.x, warp = it >> 5;
    const bool act = it < THREADS;
    int k1 = 0, l = 0;
    if (act) {
        if (LS == 1) { k1 = it / NL; l = it - k1 * NL; }
        else { l = it / 6; k1 = it - l * 6; }
    }
    float2 *b = buf + l * LS;
    float2 y0 = make_float2(0.f, 0.f);
    float ax[20], ay[20], bx[20], by[20];
    if (act) {
        y0 = b[(41 * k1) * PS];
#pragma unroll
        for (int n = 1; n <= 20; ++n) {
            const float2 p = b[(41 * k1 + n) * PS], q = b[(41 * k1 + 41 - n) * PS];
            ax[n - 1] = p.x + q.x; ay[n - 1] = p.y + q.y;
            bx[n - 1] = p.x - q.x; by[n - 1] = p.y - q.y;
        }
    } else {
#pragma unroll
        for (int n = 0; n < 20; ++n) ax[n] = ay[n] = bx[n] = by[n] = 0.f;
    }
    float s0x = y0.x, s0y = y0.y;
#pragma unroll
    for (int n = 0; n < 20; ++n) { s0x += ax[n]; s0y += ay[n]; }
    __syncthreads();   // every input read: the buffer is overwritten in place below
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    constexpr int NT = (THREADS + 127) / 128;   // tiles of 128 items
    constexpr float sg = DIR < 0 ? 1.f : -1.f;  // -DIR
#pragma unroll 1
    for (int t = 0; t < NT; ++t) {
        const bool mine = act && (warp >> 2) == t;
        if ((warp >> 2) == t) {   // the tile's warps (whole warps: .sync.aligned)
            float hi[8], lo[8];
#pragma unroll
            for (int g = 0; g < 5; ++g) {     // A_re = [a.x | -DIR b.y]
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int j = 8 * g + q;
                    const float v = j < 20 ? ax[j] : sg * by[j - 20];
                    hi[q] = tf32_hi(v);
                    lo[q] = v - hi[q];
                }
                st8(c.tmem + lane_base + COL_ARE_HI + 8 * g, hi);
                st8(c.tmem + lane_base + COL_ARE_LO + 8 * g, lo);
            }
#pragma unroll
            for (int g = 0; g < 5; ++g) {     // A_im = [a.y | DIR b.x]
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const int j = 8 * g + q;
                    const float v = j < 20 ? ay[j] : -sg * bx[j - 20];
                    hi[q] = tf32_hi(v);
                    lo[q] = v - hi[q];
                }
                st8(c.tmem + lane_base + COL_AIM_HI + 8 * g, hi);
                st8(c.tmem + lane_base + COL_AIM_LO + 8 * g, lo);
            }
            wait_st();
        }
        fence_before();
        __syncthreads();
        fence_after();
        if (it == 0) issue_tile(c);
        const bool ok = mbar_wait(c.mbar, c.phase);
        c.phase ^= 1u;
        fence_after();
        if ((warp >> 2) == t) {
            if (!ok && (it & 31) == 0) atomicExch(c.err, 1);
            float dr[8], di[8];
#pragma unroll
            for (int g = 0; g < 5; ++g) {
                ld8(c.tmem + lane_base + COL_DRE + 8 * g, dr);
                ld8(c.tmem + lane_base + COL_DIM + 8 * g, di);
                wait_ld();
                if (mine && ok) {
#pragma unroll
                    for (int q = 0; q < 8; ++q) {
                        const int k = 8 * g + q + 1;
                        b[(k1 + 6 * k) * PS] = make_float2(y0.x + dr[q], y0.y + di[q]);
                    }
                }
            }
            if (mine && ok) b[k1 * PS] = make_float2(s0x, s0y);
        }
        fence_before();
        __syncthreads();   // the tile's columns are read: the next tile may write them
    }
}

}  // namespace tc41

// ---------------------------------------------------------------------------
// y-axis transform of six spectra in place with the tensor-core 41-point
// stage (the k_y246 pass, fft246.cuh).  Shared memory: B hi | B lo (12,800
// bytes), the twiddles, and the line buffer without row padding (the B
// table takes that room; two blocks per SM stay resident, each with 256
// TMEM columns).  btab: the B table in its shared-memory byte layout.
// ---------------------------------------------------------------------------
namespace tc41 {
constexpr int PS_Y = f246::NL;
constexpr size_t y_smem_bytes() {
    return (size_t)2 * B_BYTES + (size_t)(f246::N + f246::N * PS_Y) * sizeof(float2);
}
}  // namespace tc41

template <int DIR>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_y246tc(Grid3 g, const float2 *tw_g, const float4 *btab, AxisIO<float, 6, 6> io, const double *skip, int *err) {
    using namespace f246;
    constexpr int TP = TC / 2, PS = tc41::PS_Y;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tbase;
    if (skip && *skip != 0.0) return;
    float4 *bt = reinterpret_cast<float4 *>(smem_raw);
    float2 *tw = reinterpret_cast<float2 *>(smem_raw + 2 * tc41::B_BYTES);
    float2 *buf = tw + N;
    const int warp = threadIdx.x >> 5;
    if (warp == 0) tc41::tmem_alloc(&tbase, tc41::TMEM_COLS);
    if (threadIdx.x == 0) tc41::mbar_init(&mbar);
    const int k0 = blockIdx.x * TC, i = blockIdx.y;
    const int kcnt = min(TC, g.NzC - k0);
    const long long base = (long long)i * N * g.NzC + k0;
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        for (int e = threadIdx.x; e < N * TP; e += blockDim.x) {
            const int tp = e % TP, y = e / TP;
            const int t = 2 * tp;
            float2 *dst = buf + y * PS + s * TC + t;
            const float2 *src = io.in[s] + base + (long long)y * g.NzC + t;
            if (t + 1 < kcnt) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src));
            } else {
                dst[0] = t < kcnt ? src[0] : make_float2(0.f, 0.f);
                dst[1] = make_float2(0.f, 0.f);
            }
        }
    }
    for (int e = threadIdx.x; e < 2 * tc41::B_BYTES / 16; e += blockDim.x) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(bt + e);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(btab + e));
    }
    cp_async_commit();
    load_twiddles(tw, tw_g);
    cp_async_wait_all();
    // the B table is read by the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc41::fence_before();
    __syncthreads();
    tc41::fence_after();
    tc41::Ctx c{tbase, &mbar, 0u, tc41::smem_u32(bt), tc41::smem_u32(bt) + tc41::B_BYTES, err};
    stage_a<DIR, PS, 1>(buf, tw);
    __syncthreads();
    tc41::stage_c<DIR, PS, 1>(buf, c);
#pragma unroll
    for (int s = 0; s < 6; ++s) {
        for (int e = threadIdx.x; e < N * TP; e += blockDim.x) {
            const int tp = e % TP, y = e / TP;
            const int t = 2 * tp;
            const float2 *srcs = buf + y * PS + s * TC + t;
            float2 *dst = io.out[s] + base + (long long)y * g.NzC + t;
            if (t + 1 < kcnt) *reinterpret_cast<float4 *>(dst) = *reinterpret_cast<const float4 *>(srcs);
            else if (t < kcnt) dst[0] = srcs[0];
        }
    }
    tc41::fence_before();
    __syncthreads();
    if (warp == 0) tc41::tmem_dealloc(tbase, tc41::TMEM_COLS);
}

namespace tc41 {
// per-block set-up of the tensor-core stage, called by all threads before
// the first transform: TMEM columns (warp 0), the completion barrier
// (thread 0) and the B table copied into shared memory with 16-byte
// cp.async (committed with the caller's group; after its cp.async wait the
// caller calls ready())
__device__ __forceinline__ void begin(uint32_t *tbase, uint64_t *mbar, float4 *bt, const float4 *btab) {
    if ((threadIdx.x >> 5) == 0) tmem_alloc(tbase, TMEM_COLS);
    if (threadIdx.x == 0) mbar_init(mbar);
    for (int e = threadIdx.x; e < 2 * B_BYTES / 16; e += blockDim.x) {
        const unsigned sa = (unsigned)__cvta_generic_to_shared(bt + e);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(btab + e));
    }
}
// the B table made visible to the tensor core, the TMEM base to every thread
__device__ __forceinline__ Ctx ready(uint32_t *tbase, uint64_t *mbar, float4 *bt, int *err) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    fence_after();
    return Ctx{*tbase, mbar, 0u, smem_u32(bt), smem_u32(bt) + B_BYTES, err};
}
__device__ __forceinline__ void end(uint32_t tmem) {
    fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) tmem_dealloc(tmem, TMEM_COLS);
}
// one transform of the block's NL lines: the radix-6 stage on the CUDA
// cores, the 41-point stage on the tensor cores
template <int DIR, int PS, int LS>
__device__ __forceinline__ void lines(float2 *buf, const float2 *tw, Ctx &c) {
    f246::stage_a<DIR, PS, LS>(buf, tw);
    __syncthreads();
    stage_c<DIR, PS, LS>(buf, c);
}
}  // namespace tc41

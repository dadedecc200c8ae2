// fft246.cuh — FP32 line transforms of length 246 = 6 x 41 for the grids
// whose axes are 246 long, and the three elastic-iteration passes built on
// them (y transform of six spectra, x transform + Green's operator, z
// C2R -> h_ij -> R2C).
//
// Cooley-Tukey with n = 41 n1 + n2 and k = k1 + 6 k2:
//   X[k1 + 6 k2] = sum_n2 W41^(n2 k2) W246^(n2 k1) sum_n1 x[41 n1 + n2] W6^(n1 k1)
// stage A: for each (line, n2) the 6-point DFT over n1, times W246^(n2 k1),
//          written back to the same six slots (position 41 k1 + n2);
// stage C: for each (line, k1) the 41-point DFT over n2 of positions
//          41 k1 .. 41 k1 + 40, written to positions k1 + 6 k2.
// Stage C is a direct DFT per thread using the symmetric pairing
// a_n = y_n + y_(41-n), b_n = y_n - y_(41-n):
//   X_q      = y_0 + sum a_n cos(2 pi n q / 41) + DIR i sum b_n sin(2 pi n q / 41)
//   X_(41-q) = the same with the sine sum negated,       q = 1..20,
// 1,600 fused multiply-adds per 41-point DFT with compile-time constants.
// A block holds NL lines and runs all NL * 6 stage-C items at once: each
// thread reads its 41 inputs, the block synchronises, then all write.
#pragma once

#include "fft.cuh"

namespace f246 {

constexpr int N = 246;
constexpr int NL = 48;            // lines per block: 6 spectra x TC columns, or ZR z rows x 3 field pairs
constexpr int TC = NL / 6;        // columns per block of the strided-axis passes (even: 16-byte pairs)
constexpr int ZR = NL / 3;        // rows per block of the z pass
constexpr int THREADS = NL * 6;   // one stage-C item per thread
constexpr int BLOCKS_PER_SM = 96 / NL;
// position stride of the lines-fast layout.  (With NL = 24 a warp's second
// half of stage-C reads spans two items 41 * PSTR apart, which land on
// disjoint banks when 82 * PSTR = 16 (mod 32); 24 lines per block measured
// slower than 48: 32-byte column segments and twice the per-block overhead.)
constexpr int PSTR = NL == 24 ? 24 : NL + 4;
static_assert(NL % 6 == 0 && TC % 2 == 0, "lines per block: 6 spectra x an even column count");

// stage A over NL lines; element (line l, position p) at buf[p * PS + l * LS]
template <int DIR, int PS, int LS>
__device__ __forceinline__ void stage_a(float2 *buf, const float2 *tw) {
    constexpr int ITEMS = NL * 41;
    for (int it = threadIdx.x; it < ITEMS; it += blockDim.x) {
        int l, n2;
        if (LS == 1) { n2 = it / NL; l = it - n2 * NL; }   // consecutive threads: consecutive lines
        else { l = it / 41; n2 = it - l * 41; }             // consecutive threads: consecutive positions
        float2 *b = buf + l * LS + n2 * PS;
        float2 v[6];
#pragma unroll
        for (int r = 0; r < 6; ++r) v[r] = b[41 * r * PS];
        bfly6<float, DIR>(v);
#pragma unroll
        for (int r = 1; r < 6; ++r) v[r] = twmul<DIR>(v[r], tw[n2 * r]);
#pragma unroll
        for (int r = 0; r < 6; ++r) b[41 * r * PS] = v[r];
    }
}

// stage C; contains the block barrier that separates its reads from its writes
template <int DIR, int PS, int LS>
__device__ __forceinline__ void stage_c(float2 *buf) {
    const int it = threadIdx.x;
    const bool act = it < THREADS;
    int l, k1;
    if (LS == 1) { k1 = it / NL; l = it - k1 * NL; }
    else { l = it / 6; k1 = it - l * 6; }
    if (!act) { l = 0; k1 = 0; }
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
    }
    __syncthreads();
    if (!act) return;
    {
        float sx = y0.x, sy = y0.y;
#pragma unroll
        for (int n = 0; n < 20; ++n) { sx += ax[n]; sy += ay[n]; }
        b[k1 * PS] = make_float2(sx, sy);
    }
#pragma unroll
    for (int q = 1; q <= 20; ++q) {
        float cx = 0.f, cy = 0.f, sx = 0.f, sy = 0.f;
#pragma unroll
        for (int n = 1; n <= 20; ++n) {
            const float c = (float)dft41_cos((n * q) % 41);
            const float s = (float)dft41_sin((n * q) % 41);
            cx = fmaf(ax[n - 1], c, cx);
            cy = fmaf(ay[n - 1], c, cy);
            sx = fmaf(bx[n - 1], s, sx);
            sy = fmaf(by[n - 1], s, sy);
        }
        // DIR i S with i S = (-S.y, S.x)
        const float dx = DIR < 0 ? sy : -sy, dy = DIR < 0 ? -sx : sx;
        const float rx = y0.x + cx, ry = y0.y + cy;
        b[(k1 + 6 * q) * PS] = make_float2(rx + dx, ry + dy);
        b[(k1 + 6 * (41 - q)) * PS] = make_float2(rx - dx, ry - dy);
    }
}

// full transform of the NL lines in place; all threads of the block call it
template <int DIR, int PS, int LS>
__device__ __forceinline__ void lines(float2 *buf, const float2 *tw) {
    stage_a<DIR, PS, LS>(buf, tw);
    __syncthreads();
    stage_c<DIR, PS, LS>(buf);
    __syncthreads();
}

__device__ __forceinline__ void load_twiddles(float2 *s, const float2 *g) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) s[i] = g[i];
}

// shared memory of the strided-axis passes: twiddles + 246 x PSTR elements
constexpr size_t axis_smem_bytes() { return (size_t)(N + N * PSTR) * sizeof(float2); }
// shared memory of the z pass: twiddles + NL lines of 246
constexpr size_t z_smem_bytes() { return (size_t)(N + NL * N) * sizeof(float2); }

}  // namespace f246

// ---------------------------------------------------------------------------
// y-axis transform of six spectra in place.  Block (bx, i, h): spectra
// 3 h .. 3 h + 2, columns kz = YC bx .. YC bx + YC - 1 of x-plane i; line
// (s, t) = spectrum 3 h + s, column t.  Three spectra of 16 columns (128-byte
// row segments) measured 10% faster than six of 8 (64-byte segments), with
// the same arithmetic and bitwise the same results.
// ---------------------------------------------------------------------------
namespace f246 {
constexpr int YS = 3;             // spectra per block of the y pass
constexpr int YC = NL / YS;       // columns per block of the y pass
static_assert(YC % 2 == 0, "y pass: 16-byte column pairs");
}  // namespace f246

template <int DIR>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_y246(Grid3 g, const float2 *tw_g, AxisIO<float, 6, 6> io, const double *skip) {
    if (skip && *skip != 0.0) return;
    using namespace f246;
    constexpr int TP = YC / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *buf = tw + N;
    const int k0 = blockIdx.x * YC, i = blockIdx.y, h = blockIdx.z;
    const int kcnt = min(YC, g.NzC - k0);
    const long long base = (long long)i * N * g.NzC + k0;   // (i, y = 0, k0)
    // 16-byte copies: (spectrum, y, column pair); the spectrum loop is
    // unrolled and the half picked by a select, so that every io.in index is
    // a compile-time constant (a run-time index puts the struct in local memory)
#pragma unroll
    for (int s = 0; s < YS; ++s) {
        const float2 *in = (h ? io.in[YS + s] : io.in[s]) + base;
        for (int e = threadIdx.x; e < N * TP; e += blockDim.x) {
            const int tp = e % TP, y = e / TP;
            const int t = 2 * tp;
            float2 *dst = buf + y * PSTR + s * YC + t;
            const float2 *src = in + (long long)y * g.NzC + t;
            if (t + 1 < kcnt) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src));
            } else {
                dst[0] = t < kcnt ? src[0] : make_float2(0.f, 0.f);
                dst[1] = make_float2(0.f, 0.f);
            }
        }
    }
    cp_async_commit();
    load_twiddles(tw, tw_g);
    cp_async_wait_all();
    __syncthreads();
    lines<DIR, PSTR, 1>(buf, tw);
    // the stage-C outputs are in natural order: position k of line l
#pragma unroll
    for (int s = 0; s < YS; ++s) {
        float2 *out = (h ? io.out[YS + s] : io.out[s]) + base;
        for (int e = threadIdx.x; e < N * TP; e += blockDim.x) {
            const int tp = e % TP, y = e / TP;
            const int t = 2 * tp;
            const float2 *srcs = buf + y * PSTR + s * YC + t;
            float2 *dst = out + (long long)y * g.NzC + t;
            if (t + 1 < kcnt) *reinterpret_cast<float4 *>(dst) = *reinterpret_cast<const float4 *>(srcs);
            else if (t < kcnt) dst[0] = srcs[0];
        }
    }
}

// ---------------------------------------------------------------------------
// generic strided-axis pass on the 246-point engine: NIN spectra in, an
// optional forward transform (DIN), the op's per-point apply(i, j, k, in, out)
// in place, an optional inverse transform (DOUT), NOUT spectra out.  The 48
// lines of a block are NW = max(NIN, NOUT) arrays x TC = 48 / NW columns.
// axis 1: y (block (bx, x-plane)); axis 2: x (block (bx, y-row)).  Lines
// beyond the NIN inputs are transformed too and never stored.
// ---------------------------------------------------------------------------
template <int NIN, int NOUT>
constexpr bool f246_axis_fits() {
    constexpr int NW = NIN > NOUT ? NIN : NOUT;
    return NW >= 1 && NW <= 6 && f246::NL % NW == 0 && (f246::NL / NW) % 2 == 0;
}

template <int NIN, int NOUT, int DIN, int DOUT, class Op>
__global__ void __launch_bounds__(f246::THREADS, f246::BLOCKS_PER_SM)
k_axis246(Grid3 g, int axis, const float2 *tw_g, AxisIO<float, NIN, NOUT> io, Op op, const double *skip) {
    if (skip && *skip != 0.0) return;
    using namespace f246;
    constexpr int NW = NIN > NOUT ? NIN : NOUT;
    constexpr int TCW = NL / NW, TPW = TCW / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *buf = tw + N;
    const int k0 = blockIdx.x * TCW, slab = blockIdx.y;
    const int kcnt = min(TCW, g.NzC - k0);
    long long base, es;
    if (axis == 1) { base = (long long)slab * N * g.NzC + k0; es = g.NzC; }
    else { base = (long long)slab * g.NzC + k0; es = (long long)g.Ny * g.NzC; }
#pragma unroll
    for (int s = 0; s < NIN; ++s) {
        for (int e = threadIdx.x; e < N * TPW; e += blockDim.x) {
            const int tp = e % TPW, q = e / TPW;
            const int t = 2 * tp;
            float2 *dst = buf + q * PSTR + s * TCW + t;
            const float2 *src = io.in[s] + base + (long long)q * es + t;
            if (t + 1 < kcnt) {
                const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src));
            } else {
                dst[0] = t < kcnt ? src[0] : make_float2(0.f, 0.f);
                dst[1] = make_float2(0.f, 0.f);
            }
        }
    }
    cp_async_commit();
    if (DIN != 0 || DOUT != 0) load_twiddles(tw, tw_g);
    cp_async_wait_all();
    __syncthreads();
    if (DIN != 0) lines<DIN, PSTR, 1>(buf, tw);
    if constexpr (!Op::kInplace) {
        for (int e = threadIdx.x; e < N * TCW; e += blockDim.x) {
            const int q = e / TCW, t = e % TCW;
            const int i = axis == 1 ? slab : q, j = axis == 1 ? q : slab;
            float2 vin[NIN > 0 ? NIN : 1], vout[NOUT > 0 ? NOUT : 1];
            float2 *pt = buf + q * PSTR + t;
#pragma unroll
            for (int s = 0; s < NIN; ++s) vin[s] = pt[s * TCW];
            op.apply(i, j, k0 + t, vin, vout);
#pragma unroll
            for (int s = 0; s < NOUT; ++s) pt[s * TCW] = vout[s];
        }
        __syncthreads();
    }
    if (DOUT != 0) lines<DOUT, PSTR, 1>(buf, tw);
#pragma unroll
    for (int s = 0; s < NOUT; ++s) {
        for (int e = threadIdx.x; e < N * TPW; e += blockDim.x) {
            const int tp = e % TPW, q = e / TPW;
            const int t = 2 * tp;
            const float2 *srcs = buf + q * PSTR + s * TCW + t;
            float2 *dst = io.out[s] + base + (long long)q * es + t;
            if (t + 1 < kcnt) *reinterpret_cast<float4 *>(dst) = *reinterpret_cast<const float4 *>(srcs);
            else if (t < kcnt) dst[0] = srcs[0];
        }
    }
}

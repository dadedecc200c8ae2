// fft.cuh — shared-memory mixed-radix FFT engine and 3D pass kernels.
//
// The 3D real transform of a C-order [Nx][Ny][Nz] grid is done in three
// passes, each reading and writing the whole array once:
//   z pass : real rows (contiguous, length Nz) <-> half spectra (NzC = Nz/2+1)
//   y pass : complex lines of length Ny, element stride NzC
//   x pass : complex lines of length Nx, element stride Ny*NzC
// Each pass stages a tile of lines in shared memory and runs a Stockham
// autosort FFT there (radices 8,4,2,3,5 coded, any other prime factor as a
// direct DFT stage).  The passes take functors, so pointwise physics (RHS,
// flux, eigenstrain/h_ij, stress) runs inside the z pass, and the spectral
// updates (semi-implicit filters, gradients, Green's contraction) run inside
// the x pass between the forward and the inverse x transform.
//
// Real-data trick: two real lines a, b are transformed as one complex line
// z = a + i b;  A_k = (Z_k + conj Z_{N-k})/2, B_k = (Z_k - conj Z_{N-k})/(2i).
// The inverse packs two half spectra the same way; the imaginary parts of the
// k=0 and Nyquist bins are ignored (Hermitian input), like the C2R transform
// of the reference.
#pragma once

#include <type_traits>

#include "common.cuh"
#include "rader41.cuh"

#define PFGB_MAX_STAGES 16
#define PFGB_MAX_N 1024

// Division by a run-time constant d via a multiply-high (round-up method):
// valid for every 32-bit dividend.
struct FastDiv {
    unsigned M;
    int L;
    unsigned d;
    __host__ __device__ void init(unsigned dd) {
        d = dd;
        if (d <= 1) { M = 0; L = 0; return; }
        L = 0;
        while ((1u << L) < d) ++L;
        M = (unsigned)((((unsigned long long)1 << 32) * ((1ull << L) - d)) / d + 1);
    }
    __device__ __forceinline__ unsigned div(unsigned x) const {
        if (d <= 1) return x;
        const unsigned t = __umulhi(M, x);
        return (t + ((x - t) >> 1)) >> (L - 1);
    }
};

struct StagePlan {
    int R, Ns, nb, m;          // radix, span so far, butterflies per line, twiddle stride
    FastDiv fNs, fnb;
};

struct AxisPlan {
    int n;
    int nst;
    StagePlan st[PFGB_MAX_STAGES];
};

// host: factor n into stages.  A radix-41 factor goes first (its Rader stage
// then needs no input twiddles), then 8, 6, 4, 2, 3, 5, 7, other primes.
static inline void pfgb_make_plan(int n, AxisPlan *p) {
    p->n = n;
    p->nst = 0;
    int rad[PFGB_MAX_STAGES], nr = 0;
    int m = n;
    while (m % 41 == 0 && m > 1) { rad[nr++] = 41; m /= 41; }
    while (m % 8 == 0 && m > 1) { rad[nr++] = 8; m /= 8; }
    while (m % 6 == 0 && m > 1) { rad[nr++] = 6; m /= 6; }
    while (m % 4 == 0 && m > 1) { rad[nr++] = 4; m /= 4; }
    while (m % 2 == 0 && m > 1) { rad[nr++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2)
        while (m % f == 0) { rad[nr++] = f; m /= f; }
    int Ns = 1;
    for (int s = 0; s < nr; ++s) {
        StagePlan &st = p->st[p->nst++];
        st.R = rad[s];
        st.Ns = Ns;
        st.nb = n / rad[s];
        st.m = n / (Ns * rad[s]);
        st.fNs.init((unsigned)Ns);
        st.fnb.init((unsigned)st.nb);
        Ns *= rad[s];
    }
}

// ---------------------------------------------------------------------------
// radix butterflies.  DIR = -1 forward (exp(-i..)), +1 inverse.
// ---------------------------------------------------------------------------
template <int DIR, typename T2> __device__ __forceinline__ T2 rot_mi(T2 a) {
    // forward: multiply by -i ; inverse: by +i
    return DIR < 0 ? mk2<T2>(a.y, -a.x) : mk2<T2>(-a.y, a.x);
}

template <typename T, int DIR>
__device__ __forceinline__ void bfly2(cplx_t<T> *v) {
    auto a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
template <typename T, int DIR>
__device__ __forceinline__ void bfly4(cplx_t<T> *v) {
    auto t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    auto t2 = cadd(v[1], v[3]), t3 = rot_mi<DIR>(csub(v[1], v[3]));
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
}
template <typename T, int DIR>
__device__ __forceinline__ void bfly8(cplx_t<T> *v) {
    using T2 = cplx_t<T>;
    T2 e[4] = {v[0], v[2], v[4], v[6]};
    T2 o[4] = {v[1], v[3], v[5], v[7]};
    bfly4<T, DIR>(e);
    bfly4<T, DIR>(o);
    const T r = T(0.70710678118654752440084436210485);
    // W8^1 = r(1 -+ i), W8^2 = -+i, W8^3 = r(-1 -+ i)
    T2 o1 = DIR < 0 ? mk2<T2>(r * (o[1].x + o[1].y), r * (o[1].y - o[1].x))
                    : mk2<T2>(r * (o[1].x - o[1].y), r * (o[1].y + o[1].x));
    T2 o2 = rot_mi<DIR>(o[2]);
    T2 o3 = DIR < 0 ? mk2<T2>(r * (o[3].y - o[3].x), -r * (o[3].x + o[3].y))
                    : mk2<T2>(-r * (o[3].x + o[3].y), r * (o[3].x - o[3].y));
    v[0] = cadd(e[0], o[0]); v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);   v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);   v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);   v[7] = csub(e[3], o3);
}
template <typename T, int DIR>
__device__ __forceinline__ void bfly3(cplx_t<T> *v) {
    using T2 = cplx_t<T>;
    const T s3 = T(0.86602540378443864676372317075294);
    T2 a = v[0], s = cadd(v[1], v[2]), d = csub(v[1], v[2]);
    T2 m = mk2<T2>(a.x - T(0.5) * s.x, a.y - T(0.5) * s.y);
    T2 r = rot_mi<DIR>(cscale(d, s3));
    v[0] = cadd(a, s);
    v[1] = cadd(m, r);
    v[2] = csub(m, r);
}
template <typename T, int DIR>
__device__ __forceinline__ void bfly5(cplx_t<T> *v) {
    using T2 = cplx_t<T>;
    const T c1 = T(0.30901699437494742410229341718282);
    const T c2 = T(-0.80901699437494742410229341718282);
    const T s1 = T(0.95105651629515357211643933337938);
    const T s2 = T(0.58778525229247312916870595463907);
    T2 x0 = v[0];
    T2 a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    T2 a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    T2 p1 = mk2<T2>(x0.x + c1 * a1.x + c2 * a2.x, x0.y + c1 * a1.y + c2 * a2.y);
    T2 p2 = mk2<T2>(x0.x + c2 * a1.x + c1 * a2.x, x0.y + c2 * a1.y + c1 * a2.y);
    T2 q1 = rot_mi<DIR>(mk2<T2>(s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y));
    T2 q2 = rot_mi<DIR>(mk2<T2>(s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y));
    v[0] = mk2<T2>(x0.x + a1.x + a2.x, x0.y + a1.y + a2.y);
    v[1] = cadd(p1, q1);
    v[4] = csub(p1, q1);
    v[2] = cadd(p2, q2);
    v[3] = csub(p2, q2);
}

// Asynchronous global->shared element copy (cp.async, sm_80+): all of a
// thread's tile loads are in flight at once.  `valid == false` zero-fills
// (source size 0; the source address is clamped to a valid one).
template <typename T2>
__device__ __forceinline__ void cp_async_elem(T2 *smem, const T2 *gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(T2) == 16) {
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0));
    } else {
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 8 : 0));
    }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// twiddle w = W_n^e (table holds the forward roots); inverse uses conj
template <int DIR, typename T2>
__device__ __forceinline__ T2 twmul(T2 a, T2 w) {
    return DIR < 0 ? cmul(a, w) : cmulconj(a, w);
}

template <typename T, int DIR>
__device__ __forceinline__ void bfly6(cplx_t<T> *v) {
    // 6 = 2 x 3: E = DFT3(x0,x2,x4), O = DFT3(x1,x3,x5), X_k = E_k + W6^k O_k
    using T2 = cplx_t<T>;
    T2 e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
    bfly3<T, DIR>(e);
    bfly3<T, DIR>(o);
    const T h = T(0.5), s3 = T(0.86602540378443864676372317075294);
    // W6^1 = (1/2, -+ s3), W6^2 = (-1/2, -+ s3)
    const T sg = DIR < 0 ? -s3 : s3;
    T2 o1 = mk2<T2>(h * o[1].x - sg * o[1].y, h * o[1].y + sg * o[1].x);
    T2 o2 = mk2<T2>(-h * o[2].x - sg * o[2].y, -h * o[2].y + sg * o[2].x);
    v[0] = cadd(e[0], o[0]); v[3] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);   v[4] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);   v[5] = csub(e[2], o2);
}

// ---------------------------------------------------------------------------
// Radix-41 stage by Rader's algorithm, 8 lanes per 41-point DFT.
//   X_0 = sum x ;  X_{7^q} = x_0 + (a (*) b)_q,  a_p = x_{6^p}  (mod 41)
// The length-40 cyclic convolution is IFFT40(FFT40(a) . B) with
// B = FFT40(b)/40 (rader41.cuh).  FFT40 = 5 x 8: lane t (0..7) owns
// a[t + 8m], m = 0..4, does the 5-point DFTs in registers, the W40^{t k1}
// twiddles, and the 8-point DFTs run across the 8 lanes with shuffles
// (decimation in frequency forward -> bit-reversed lanes, decimation in time
// inverse -> natural lanes).  Index maps: 6^(t+8m) = 6^t 10^m, 7^(t+8m) =
// 7^t 37^m (mod 41).
// ---------------------------------------------------------------------------
template <typename T> struct RaderTab;
template <> struct RaderTab<float> {
    static __device__ __forceinline__ float2 B(int dir, int k) { return dir < 0 ? c_rader41_BF_f[k] : c_rader41_BI_f[k]; }
};
template <> struct RaderTab<double> {
    static __device__ __forceinline__ double2 B(int dir, int k) { return dir < 0 ? c_rader41_BF_d[k] : c_rader41_BI_d[k]; }
};

template <typename T2>
__device__ __forceinline__ T2 shfl_x(T2 v, int m, unsigned mask) {
    v.x = __shfl_xor_sync(mask, v.x, m, 8);
    v.y = __shfl_xor_sync(mask, v.y, m, 8);
    return v;
}

template <typename T, int DIR>
__device__ void stage_rader41(const cplx_t<T> *src, cplx_t<T> *dst, const StagePlan &st,
                              const cplx_t<T> *tw, int nl, int sp, int sl, bool lineFast, const FastDiv &fnl) {
    using T2 = cplx_t<T>;
    const int nb = st.nb, Ns = st.Ns, m = st.m;
    const FastDiv fnb = st.fnb, fNs = st.fNs;     // register copies
    const int t = threadIdx.x & 7;
    const int group = threadIdx.x >> 3, ngroups = blockDim.x >> 3;
    const unsigned gmask = 0xffu << (threadIdx.x & 24);
    const int brt = ((t & 1) << 2) | (t & 2) | ((t & 4) >> 2);
    // per-lane constants: W40^{t k1}, B[k1 + 5 br(t)], butterfly signs/twiddles,
    // and the shared-memory offsets of the lane's 5 inputs and 5 outputs
    T2 W[5], Bk[5];
#pragma unroll
    for (int k1 = 0; k1 < 5; ++k1) {
        T sn, cs;
        if constexpr (sizeof(T) == 4) sincospif(-2.0f * (float)(t * k1) / 40.0f, &sn, &cs);
        else sincospi(-2.0 * (double)(t * k1) / 40.0, &sn, &cs);
        W[k1] = mk2<T2>(cs, sn);
        Bk[k1] = RaderTab<T>::B(DIR, k1 + 5 * brt);
    }
    const T r = T(0.70710678118654752440084436210485);
    const int p4 = t & 3, p2 = t & 1;
    // forward twiddles of the lane's DIF butterflies (W8^{p4}, W4^{p2}); the
    // lower lane of a pair uses 1 and sign +1, the upper one f and sign -1
    const T2 one = mk2<T2>(T(1), T(0));
    const T2 f4 = p4 == 0 ? one : p4 == 1 ? mk2<T2>(r, -r) : p4 == 2 ? mk2<T2>(T(0), T(-1)) : mk2<T2>(-r, -r);
    const T2 f2 = p2 == 0 ? one : mk2<T2>(T(0), T(-1));
    const T s4 = (t & 4) ? T(-1) : T(1), s2 = (t & 2) ? T(-1) : T(1), s1 = (t & 1) ? T(-1) : T(1);
    const T2 w4 = (t & 4) ? f4 : one, w2 = (t & 2) ? f2 : one;
    // inverse (DIT) twiddles W8^{+p4}, W4^{+p2} applied by the upper lane
    const T2 c4 = mk2<T2>(f4.x, -f4.y), c2 = mk2<T2>(f2.x, -f2.y);
    int inoff[5], nidx[5], outoff[5];
    {
        int n = 1, o = 1;
        for (int i = 0; i < t; ++i) { n = (n * 6) % 41; o = (o * 7) % 41; }
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            nidx[q] = n;
            inoff[q] = n * nb * sp;
            outoff[q] = o * Ns * sp;
            n = (n * 10) % 41;
            o = (o * 37) % 41;
        }
    }
    const int items = nl * nb;
    for (int it = group; it < items; it += ngroups) {
        int j, l;
        if (lineFast) { l = (int)fnb.div((unsigned)it); j = it - l * nb; }
        else { j = (int)fnl.div((unsigned)it); l = it - j * nl; }
        const int jq = (int)fNs.div((unsigned)j);
        const int k = j - jq * Ns;
        const T2 *sb = src + l * sl + j * sp;
        T2 v[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            T2 x = sb[inoff[q]];
            if (Ns > 1) x = twmul<DIR>(x, tw[nidx[q] * k * m]);
            v[q] = x;
        }
        const T2 x0 = sb[0];
        // X_0 = x_0 + sum over the 40 permuted inputs
        T2 s = cadd(cadd(cadd(v[0], v[1]), cadd(v[2], v[3])), v[4]);
        s = cadd(s, shfl_x(s, 1, gmask));
        s = cadd(s, shfl_x(s, 2, gmask));
        s = cadd(s, shfl_x(s, 4, gmask));
        // forward FFT40 of a: in-lane DFT5, twiddle, cross-lane DFT8 (DIF)
        bfly5<T, -1>(v);
#pragma unroll
        for (int q = 1; q < 5; ++q) v[q] = cmul(v[q], W[q]);
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            // DIF: lower a + b, upper (a - b) w  ==  (partner + sign * own) * w_lane
            T2 u = shfl_x(v[q], 4, gmask);
            v[q] = cmul(mk2<T2>(u.x + s4 * v[q].x, u.y + s4 * v[q].y), w4);
            u = shfl_x(v[q], 2, gmask);
            v[q] = cmul(mk2<T2>(u.x + s2 * v[q].x, u.y + s2 * v[q].y), w2);
            u = shfl_x(v[q], 1, gmask);
            v[q] = mk2<T2>(u.x + s1 * v[q].x, u.y + s1 * v[q].y);
            v[q] = cmul(v[q], Bk[q]);
            // inverse DIT (bit-reversed in, natural out): the upper lane sends
            // w b; lower: a + (w b), upper: a - (w b)
            T2 sv = v[q];                                  // span 1: w = 1
            u = shfl_x(sv, 1, gmask);
            v[q] = (t & 1) ? csub(u, sv) : cadd(v[q], u);
            sv = (t & 2) ? cmul(v[q], c2) : v[q];
            u = shfl_x(sv, 2, gmask);
            v[q] = (t & 2) ? csub(u, sv) : cadd(v[q], u);
            sv = (t & 4) ? cmul(v[q], c4) : v[q];
            u = shfl_x(sv, 4, gmask);
            v[q] = (t & 4) ? csub(u, sv) : cadd(v[q], u);
        }
#pragma unroll
        for (int q = 1; q < 5; ++q) v[q] = cmulconj(v[q], W[q]);
        bfly5<T, +1>(v);
        // outputs X[7^(t+8m)] = x0 + c[t+8m]
        T2 *db = dst + l * sl + (jq * Ns * 41 + k) * sp;
#pragma unroll
        for (int q = 0; q < 5; ++q) db[outoff[q]] = cadd(x0, v[q]);
        if (t == 0) db[0] = cadd(x0, s);
    }
}

// one Stockham stage of compile-time radix R: each work item is one
// butterfly (R inputs twiddled, R-point DFT in registers, R outputs)
template <typename T, int DIR, int R>
__device__ __forceinline__ void stage_bfly(const cplx_t<T> *src, cplx_t<T> *dst, const StagePlan &st,
                                           const cplx_t<T> *tw, int nl, int sp, int sl, bool lineFast,
                                           const FastDiv &fnl) {
    using T2 = cplx_t<T>;
    const int nb = st.nb, Ns = st.Ns, m = st.m;
    const FastDiv fnb = st.fnb, fNs = st.fNs;     // register copies
    const int work = nl * nb;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
        int j, l;
        if (lineFast) { l = (int)fnb.div((unsigned)w); j = w - l * nb; }
        else { j = (int)fnl.div((unsigned)w); l = w - j * nl; }
        const int jq = (int)fNs.div((unsigned)j);
        const int k = j - jq * Ns;
        T2 v[R];
        const T2 *sb = src + l * sl;
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = sb[(j + r * nb) * sp];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = twmul<DIR>(v[r], tw[r * k * m]);
        }
        if constexpr (R == 2) bfly2<T, DIR>(v);
        else if constexpr (R == 3) bfly3<T, DIR>(v);
        else if constexpr (R == 4) bfly4<T, DIR>(v);
        else if constexpr (R == 5) bfly5<T, DIR>(v);
        else if constexpr (R == 6) bfly6<T, DIR>(v);
        else bfly8<T, DIR>(v);
        T2 *db = dst + l * sl;
        const int base = jq * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) db[(base + r * Ns) * sp] = v[r];
    }
}

// direct DFT stage for any other radix: one output per work item,
// out_q = sum_r x_r W_n^{r (k m + q n/R)}  (exponent mod n)
template <typename T, int DIR>
__device__ void stage_direct(const cplx_t<T> *src, cplx_t<T> *dst, const StagePlan &st, int n,
                             const cplx_t<T> *tw, int nl, int sp, int sl, bool lineFast, const FastDiv &fnl) {
    using T2 = cplx_t<T>;
    const int R = st.R, nb = st.nb, Ns = st.Ns, m = st.m;
    const FastDiv fnb = st.fnb, fNs = st.fNs;
    const int work = nl * n;
    for (int w = threadIdx.x; w < work; w += blockDim.x) {
        int o, l;
        if (lineFast) { l = w / n; o = w - l * n; } else { o = (int)fnl.div((unsigned)w); l = w - o * nl; }
        const int q = (int)fnb.div((unsigned)o);
        const int j = o - q * nb;
        const int jq = (int)fNs.div((unsigned)j);
        const int k = j - jq * Ns;
        int e = k * m + q * nb;
        if (e >= n) e -= n;
        const T2 *sb = src + l * sl;
        T ar = 0, ai = 0;
        int idx = 0;
        for (int r = 0; r < R; ++r) {
            T2 x = sb[(j + r * nb) * sp];
            T2 t = tw[idx];
            if (DIR < 0) { ar += x.x * t.x - x.y * t.y; ai += x.x * t.y + x.y * t.x; }
            else { ar += x.x * t.x + x.y * t.y; ai += x.y * t.x - x.x * t.y; }
            idx += e;
            if (idx >= n) idx -= n;
        }
        dst[l * sl + (jq * Ns * R + k + q * Ns) * sp] = mk2<T2>(ar, ai);
    }
}

// ---------------------------------------------------------------------------
// fft_lines: transform nl lines of length p.n held in shared memory.
// Element (line l, position q) lives at buf[q*sp + l*sl].  Stockham stages
// alternate between `a` and `b`; returns the buffer holding the result.
// lineFast: consecutive threads walk butterflies of one line (sp == 1);
// otherwise consecutive threads walk lines (sl == 1).
// Must be called by all threads of the block; ends with __syncthreads().
// ---------------------------------------------------------------------------
template <typename T, int DIR>
__device__ __forceinline__ cplx_t<T> *fft_lines(cplx_t<T> *a, cplx_t<T> *b, const AxisPlan &p,
                                                const cplx_t<T> *tw, int nl, int sp, int sl, bool lineFast) {
    using T2 = cplx_t<T>;
    FastDiv fnl;
    fnl.init((unsigned)nl);
    T2 *src = a, *dst = b;
    for (int s = 0; s < p.nst; ++s) {
        const StagePlan st = p.st[s];
        switch (st.R) {
            case 2: stage_bfly<T, DIR, 2>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 3: stage_bfly<T, DIR, 3>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 4: stage_bfly<T, DIR, 4>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 5: stage_bfly<T, DIR, 5>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 6: stage_bfly<T, DIR, 6>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 8: stage_bfly<T, DIR, 8>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            case 41: stage_rader41<T, DIR>(src, dst, st, tw, nl, sp, sl, lineFast, fnl); break;
            default: stage_direct<T, DIR>(src, dst, st, p.n, tw, nl, sp, sl, lineFast, fnl); break;
        }
        __syncthreads();
        T2 *t = src; src = dst; dst = t;
    }
    return src;
}

// load the twiddle table of length n into shared memory
template <typename T>
__device__ __forceinline__ void load_tw(cplx_t<T> *s, const cplx_t<T> *g, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) s[i] = g[i];
}

// 3D grid description passed to every pass kernel
struct Grid3 {
    int Nx, Ny, Nz, NzC;
    long long N, Nk;
};

// ---------------------------------------------------------------------------
// Strided axis pass (y or x).  A block owns TK consecutive kz columns of one
// (i) slab (y pass) or one (j) slab (x pass): lines of length n, element
// stride `es`.  All NIN arrays of the tile sit interleaved in one shared
// buffer (row q holds NIN*TK values, array-major, padded by one) and are
// transformed together by a single batched FFT with direction DIN (0 =
// none); op.apply(i, j, k, vin, vout) combines them point by point; the NOUT
// outputs are transformed together with DOUT (0 = none) and stored.
// ---------------------------------------------------------------------------
template <typename T, int NIN, int NOUT>
struct AxisIO {
    const cplx_t<T> *in[NIN > 0 ? NIN : 1];
    cplx_t<T> *out[NOUT > 0 ? NOUT : 1];
};

template <int NIN, int NOUT> constexpr int axis_width() { return NIN > NOUT ? NIN : NOUT; }

template <typename T, int NIN, int NOUT, int DIN, int DOUT, class Op>
__global__ void __launch_bounds__(256)
k_axis_pass(Grid3 g, int axis, AxisPlan plan, const cplx_t<T> *tw_g, int TK,
            AxisIO<T, NIN, NOUT> io, Op op, const double *skip) {
    if (skip && *skip != 0.0) return;   // a finished elastic iteration: launched ahead, nothing to do
    using T2 = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *sm = reinterpret_cast<T2 *>(smem_raw);
    constexpr int NW = axis_width<NIN, NOUT>();
    const int n = plan.n;
    const int SPI = NIN * TK + 1, SPO = NOUT * TK + 1;   // padded row strides
    const int buf = n * (NW * TK + 1);
    T2 *tw = sm;
    T2 *A = sm + n, *B = A + buf;
    constexpr bool INPL = Op::kInplace;   // identity op: outputs are the inputs

    const int k0 = blockIdx.x * TK;
    const int slab = blockIdx.y;       // i for the y pass, j for the x pass
    long long base, es;
    if (axis == 1) { base = (long long)slab * g.Ny * g.NzC + k0; es = g.NzC; }
    else { base = (long long)slab * g.NzC + k0; es = (long long)g.Ny * g.NzC; }
    const int kcnt = min(TK, g.NzC - k0);
    const int lgTK = __ffs(TK) - 1;    // TK is a power of two

    if (DIN != 0 || DOUT != 0) load_tw<T>(tw, tw_g, n);
#pragma unroll
    for (int a = 0; a < NIN; ++a) {
        for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
            const int q = e >> lgTK, l = e & (TK - 1);
            const bool ok = l < kcnt;
            cp_async_elem(&A[q * SPI + a * TK + l], io.in[a] + (ok ? base + q * es + l : base), ok);
        }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    T2 *cur = A, *oth = B;
    if (DIN != 0) {
        T2 *r = fft_lines<T, DIN>(cur, oth, plan, tw, NIN * TK, SPI, 1, false);
        if (r != cur) { oth = cur; cur = r; }
    }
    int SP = SPI;
    if constexpr (!INPL) {
        for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
            const int q = e >> lgTK, l = e & (TK - 1);
            const int k = k0 + l;
            const int i = (axis == 1) ? slab : q;
            const int j = (axis == 1) ? q : slab;
            T2 vin[NIN > 0 ? NIN : 1], vout[NOUT > 0 ? NOUT : 1];
#pragma unroll
            for (int a = 0; a < NIN; ++a) vin[a] = cur[q * SPI + a * TK + l];
            op.apply(i, j, k, vin, vout);
#pragma unroll
            for (int a = 0; a < NOUT; ++a) oth[q * SPO + a * TK + l] = vout[a];
        }
        __syncthreads();
        T2 *t = cur; cur = oth; oth = t;
        SP = SPO;
    }
    if (DOUT != 0) {
        T2 *r = fft_lines<T, DOUT>(cur, oth, plan, tw, NOUT * TK, SP, 1, false);
        if (r != cur) { oth = cur; cur = r; }
    }
#pragma unroll
    for (int a = 0; a < NOUT; ++a) {
        for (int e = threadIdx.x; e < n * TK; e += blockDim.x) {
            const int q = e >> lgTK, l = e & (TK - 1);
            if (l < kcnt) io.out[a][base + q * es + l] = cur[q * SP + a * TK + l];
        }
    }
}

// ops of the z pass may declare kBatch > 1 with a Pre type, fetch(cell, pre)
// and point_with(cell, pre, in, out, acc): their global reads are then
// issued for kBatch cells of a thread at once
template <class Op, class = void>
struct op_batch { static constexpr int value = 1; };
template <class Op>
struct op_batch<Op, std::void_t<decltype(Op::kBatch)>> { static constexpr int value = Op::kBatch; };

// identity op for plain axis transforms
template <typename T, int NF>
struct OpCopy {
    static constexpr bool kInplace = true;
    __device__ __forceinline__ void apply(int, int, int, const cplx_t<T> *vin, cplx_t<T> *vout) const {
#pragma unroll
        for (int a = 0; a < NF; ++a) vout[a] = vin[a];
    }
};

// ---------------------------------------------------------------------------
// z pass: R consecutive rows per block.  Inputs: NFI half spectra per row
// (op.load_spec), inverse-transformed to real (C2R, unnormalised); then
// op.point(cell, in[NFI], out[NFO]) per cell; then NFO real fields are
// forward-transformed (R2C) and handed to op.store_spec(row, kz, v[NFO]).
// NFI = 0 makes it a pure R2C pass with a pointwise producer, NFO = 0 a pure
// C2R pass with a pointwise consumer.
// Real lines are paired (line 2p -> real part, 2p+1 -> imaginary part of
// complex line p); line index = row * NF + field.
// ---------------------------------------------------------------------------
// Reduction hook of the z pass: an op declares `struct Acc` with
// kActive, identity(), combine(a, b) and shuffle-able members (reduced with
// warp shuffles + shared memory, deterministic for a fixed launch shape).
struct NoAcc {
    static constexpr bool kActive = false;
    __device__ static NoAcc identity() { return NoAcc(); }
};

template <class Acc>
__device__ void block_reduce_acc(Acc &a) {
    __shared__ Acc red[32];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) a = Acc::combine(a, Acc::shfl_down(a, off));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = a;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        a = (lane < nw) ? red[lane] : Acc::identity();
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) a = Acc::combine(a, Acc::shfl_down(a, off));
    }
}

template <typename T, int NFI, int NFO, class Op>
__global__ void __launch_bounds__(256)
k_zpass(Grid3 g, AxisPlan plan, const cplx_t<T> *tw_g, int R, Op op, const double *skip) {
    if (skip && *skip != 0.0) return;
    using T2 = cplx_t<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *sm = reinterpret_cast<T2 *>(smem_raw);
    const int n = g.Nz, nc = g.NzC;
    T2 *tw = sm;
    T2 *ws = sm + n;
    const int PI_ = (NFI > 0) ? (R * NFI + 1) / 2 : 0;
    const int PO_ = (NFO > 0) ? (R * NFO + 1) / 2 : 0;
    // NFI == NFO: the pointwise stage runs in place on the C2R result (same
    // line layout), so two buffers suffice
    constexpr bool SAME = (NFI == NFO);
    T2 *inA = ws, *inB = ws + PI_ * n;
    T2 *outA = SAME ? nullptr : ws + 2 * PI_ * n, *outB = SAME ? nullptr : outA + PO_ * n;
    const long long row0 = (long long)blockIdx.x * R;
    const long long nrows = (long long)g.Nx * g.Ny;
    const int rcnt = (int)min((long long)R, nrows - row0);
    load_tw<T>(tw, tw_g, n);

    auto pack = [&](int p, int k, T2 A, T2 B) {
        if (k == 0 || 2 * k == n) { A.y = T(0); B.y = T(0); }
        // Z_k = A_k + i B_k ; Z_{n-k} = conj(A_k) + i conj(B_k)
        inA[p * n + k] = mk2<T2>(A.x - B.y, A.y + B.x);
        if (k > 0 && 2 * k != n) inA[p * n + (n - k)] = mk2<T2>(A.x + B.y, B.x - A.y);
    };
    if (NFI > 0 && (NFI % 2) == 0) {
        // even field count: the pairs of a row are (f0,f1), (f2,f3), ...;
        // each (row, k) is loaded once
        for (int e = threadIdx.x; e < R * nc; e += blockDim.x) {
            const int rr = e / nc, k = e - rr * nc;
            T2 v[NFI > 0 ? NFI : 1];
            if (rr < rcnt) op.load_spec(row0 + rr, k, v);
            else {
#pragma unroll
                for (int f = 0; f < NFI; ++f) v[f] = mk2<T2>(T(0), T(0));
            }
#pragma unroll
            for (int f = 0; f < NFI / 2; ++f) pack(rr * (NFI / 2) + f, k, v[2 * f], v[2 * f + 1]);
        }
        __syncthreads();
        T2 *r = fft_lines<T, +1>(inA, inB, plan, tw, PI_, 1, n, true);
        if (r != inA) { inB = inA; inA = r; }
    } else if (NFI > 0) {
        // pack pairs of half spectra into full complex spectra
        for (int e = threadIdx.x; e < PI_ * nc; e += blockDim.x) {
            const int p = e / nc, k = e - p * nc;
            T2 A = mk2<T2>(T(0), T(0)), B = mk2<T2>(T(0), T(0));
            const int la = 2 * p, lb = 2 * p + 1;
            const int ra = la / (NFI > 0 ? NFI : 1), fa = la - ra * (NFI > 0 ? NFI : 1);
            const int rb = lb / (NFI > 0 ? NFI : 1), fb = lb - rb * (NFI > 0 ? NFI : 1);
            T2 v[NFI > 0 ? NFI : 1];
            if (ra < rcnt) {
                op.load_spec(row0 + ra, k, v);
                A = v[fa];
                if (rb == ra) B = v[fb];
            }
            if (rb != ra && rb < rcnt) {
                op.load_spec(row0 + rb, k, v);
                B = v[fb];
            }
            pack(p, k, A, B);
        }
        __syncthreads();
        T2 *r = fft_lines<T, +1>(inA, inB, plan, tw, PI_, 1, n, true);
        if (r != inA) { inB = inA; inA = r; }
    }
    if constexpr (SAME) { outA = inA; outB = inB; }
    // pointwise stage
    typename Op::Acc acc = Op::Acc::identity();
    auto cell_step = [&](int e, auto &&pointf) {
        const int r = e / n, z = e - r * n;
        if (r >= rcnt) {
            if (NFO > 0) {
#pragma unroll
                for (int f = 0; f < NFO; ++f) {
                    const int l = r * NFO + f;
                    T *dst = reinterpret_cast<T *>(&outA[(l >> 1) * n + z]);
                    dst[l & 1] = T(0);
                }
            }
            return;
        }
        T vi[NFI > 0 ? NFI : 1], vo[NFO > 0 ? NFO : 1];
#pragma unroll
        for (int f = 0; f < NFI; ++f) {
            const int l = r * NFI + f;
            const T *src = reinterpret_cast<const T *>(&inA[(l >> 1) * n + z]);
            vi[f] = src[l & 1];
        }
        pointf((row0 + r) * n + z, vi, vo);
#pragma unroll
        for (int f = 0; f < NFO; ++f) {
            const int l = r * NFO + f;
            T *dst = reinterpret_cast<T *>(&outA[(l >> 1) * n + z]);
            dst[l & 1] = vo[f];
        }
    };
    constexpr int B = op_batch<Op>::value;
    if constexpr (B > 1) {
        // the op's global reads of B cells go out together before any of
        // their stores (an op that reads and writes the same field cannot
        // have them reordered by the compiler)
        for (int e0 = threadIdx.x; e0 < R * n; e0 += B * blockDim.x) {
            typename Op::Pre pre[B];
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int e = e0 + b * blockDim.x;
                const int r = e / n;
                if (e < R * n && r < rcnt) op.fetch((row0 + r) * n + (e - r * n), pre[b]);
            }
#pragma unroll
            for (int b = 0; b < B; ++b) {
                const int e = e0 + b * blockDim.x;
                if (e < R * n)
                    cell_step(e, [&](long long cell, const T *vi, T *vo) { op.point_with(cell, pre[b], vi, vo, acc); });
            }
        }
    } else {
        for (int e = threadIdx.x; e < R * n; e += blockDim.x)
            cell_step(e, [&](long long cell, const T *vi, T *vo) { op.point(cell, vi, vo, acc); });
    }
    if constexpr (Op::Acc::kActive) {
        block_reduce_acc(acc);
        if (threadIdx.x == 0) op.finish(blockIdx.x, acc);
    }
    if (NFO > 0) {
        // odd line count: zero the unused imaginary line
        if ((R * NFO) & 1) {
            const int l = R * NFO;
            for (int z = threadIdx.x; z < n; z += blockDim.x) {
                T *dst = reinterpret_cast<T *>(&outA[(l >> 1) * n + z]);
                dst[1] = T(0);
            }
        }
        __syncthreads();
        T2 *r = fft_lines<T, -1>(outA, outB, plan, tw, PO_, 1, n, true);
        if (r != outA) { outB = outA; outA = r; }
        // unpack and store: per (row, kz) gather all NFO fields
        for (int e = threadIdx.x; e < rcnt * nc; e += blockDim.x) {
            const int rr = e / nc, k = e - rr * nc;
            T2 v[NFO > 0 ? NFO : 1];
#pragma unroll
            for (int f = 0; f < NFO; ++f) {
                const int l = rr * NFO + f, p = l >> 1;
                const T2 Zk = outA[p * n + k];
                const T2 Zm = outA[p * n + (k == 0 ? 0 : n - k)];
                // A_k = (Z_k + conj Z_-k)/2 ; B_k = (Z_k - conj Z_-k)/(2i)
                if ((l & 1) == 0) v[f] = mk2<T2>(T(0.5) * (Zk.x + Zm.x), T(0.5) * (Zk.y - Zm.y));
                else v[f] = mk2<T2>(T(0.5) * (Zk.y + Zm.y), T(0.5) * (Zm.x - Zk.x));
            }
            op.store_spec(row0 + rr, k, v);
        }
    } else {
        __syncthreads();
    }
}

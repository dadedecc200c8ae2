// common.cuh — shared device/host helpers of the pfgb library.
//
// Real type T is double (plain FP64 path) or float (FP32 fields).  Complex
// values are T2 = double2 / float2 with .x = re, .y = im.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/pfgb.h"

#ifndef PFGB_PI
#define PFGB_PI 3.14159265358979323846
#endif

#define PFGB_HD __host__ __device__ __forceinline__

template <typename T> struct cplx_of;
template <> struct cplx_of<double> { using type = double2; };
template <> struct cplx_of<float> { using type = float2; };
template <typename T> using cplx_t = typename cplx_of<T>::type;

template <typename T2> PFGB_HD T2 mk2(decltype(T2::x) a, decltype(T2::x) b) { T2 r; r.x = a; r.y = b; return r; }
template <typename T2> PFGB_HD T2 cadd(T2 a, T2 b) { return mk2<T2>(a.x + b.x, a.y + b.y); }
template <typename T2> PFGB_HD T2 csub(T2 a, T2 b) { return mk2<T2>(a.x - b.x, a.y - b.y); }
template <typename T2> PFGB_HD T2 cmul(T2 a, T2 b) { return mk2<T2>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <typename T2> PFGB_HD T2 cmulconj(T2 a, T2 b) { return mk2<T2>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
template <typename T2, typename S> PFGB_HD T2 cscale(T2 a, S s) { return mk2<T2>(a.x * s, a.y * s); }
// multiply by i*s  (i s (a + ib) = -s b + i s a)
template <typename T2, typename S> PFGB_HD T2 cmul_is(T2 a, S s) { return mk2<T2>(-a.y * s, a.x * s); }

// ---------------------------------------------------------------------------
// Phase functions (same polynomials as phase_functions.h:7-56)
// ---------------------------------------------------------------------------
template <typename T> PFGB_HD T pf_h(T p) { T p2 = p * p, p3 = p2 * p; return p3 * (T(6) * p2 - T(15) * p + T(10)); }
template <typename T> PFGB_HD T pf_hp(T p) { T p2 = p * p; return T(30) * p2 * (T(1) - p) * (T(1) - p); }
template <typename T> PFGB_HD T pf_g(T p) { return p * p * (T(1) - p) * (T(1) - p); }
template <typename T> PFGB_HD T pf_gp(T p) { return T(2) * p * (T(1) - p) * (T(1) - T(2) * p); }
template <typename T> PFGB_HD T clamp01(T v) { return v < T(0) ? T(0) : (v > T(1) ? T(1) : v); }
// upper clamp 1 - e, kept below 1: in float, 1 - e rounds to 1 for e below
// 2^-25 (the reference's 1e-8 / 1e-12 guards), which would let log(1 - x)
// and 1 / (1 - x) reach infinity; the largest float below 1 is used then
template <typename T> PFGB_HD T one_minus_eps(T e) {
    const T r = T(1) - e;
    return r < T(1) ? r : T(1) - T(sizeof(T) == 4 ? 5.9604644775390625e-8 : 1.1102230246251565e-16);
}
template <typename T> PFGB_HD T clamp_eps(T v, T e) {
    const T hi = one_minus_eps(e);
    return v < e ? e : (v > hi ? hi : v);
}

// ---------------------------------------------------------------------------
// Thermodynamics.  The model (thermo_utils.h:248-579): SGTE unary Gibbs
// energies of Pb, Ag, Te, compound energies G_PbTe, G_Ag2Te, a regular
// solution with L(T) = 41212.9 - 18.05 T, optional convex extrapolation
// above x = 0.09, energies divided by mu_reference_scale.
//
// For a fixed temperature every quantity the kernels need reduces to a few
// constants: mu_A(x) = (G_A + RT ln(1-x) + L x^2) / s,
//            mu_B(x) = (G_B + RT ln x + L (1-x)^2) / s.
// ThermoConst holds those constants, computed once on the host in FP64;
// FP32 kernels receive a float copy (ThermoConstT<float>) so that every
// constant is a plain operand of their arithmetic.
// ---------------------------------------------------------------------------
template <typename S>
struct ThermoConstT {
    S GA_s, GB_s;          // G_PbTe / s, G_Ag2Te / s
    S RT_s, L_s;           // R T / s, L(T) / s
    int convex;            // thermo_convex_extrapolation_enabled
    // convex-extrapolation anchors at xc = 0.09: offsets (mu - G_s) and
    // slopes, already divided by s
    S muA_c, dmuA_c, muB_c, dmuB_c;
    S Kpen_s;              // 5000 / s
    S ddmu_c;              // dmuB_c - dmuA_c, formed in FP64
};
using ThermoConst = ThermoConstT<double>;

template <typename S>
ThermoConstT<S> thermo_as(const ThermoConst &c) {
    ThermoConstT<S> t;
    t.GA_s = S(c.GA_s); t.GB_s = S(c.GB_s); t.RT_s = S(c.RT_s); t.L_s = S(c.L_s);
    t.convex = c.convex;
    t.muA_c = S(c.muA_c); t.dmuA_c = S(c.dmuA_c); t.muB_c = S(c.muB_c); t.dmuB_c = S(c.dmuB_c);
    t.Kpen_s = S(c.Kpen_s); t.ddmu_c = S(c.ddmu_c);
    return t;
}

#define PFGB_RGAS 8.31446261815324
#define PFGB_XC_CONVEX 0.09

// Host FP64 evaluation of the SGTE expressions (used to build ThermoConst
// and the derived mu0_compound; same coefficients as thermo_utils.h:280-316).
double pfgb_host_G_PbTe(double T);
double pfgb_host_G_Ag2Te(double T);
void pfgb_thermo_const(double T, double scale, int convex, ThermoConst *tc);

// Chemical potentials split as mu = G_s + off: the large compound constant
// G_s (known exactly on the host) is kept apart from the composition-
// dependent part, so FP32 kernels can form differences such as mu_B - mu_A or
// mu0 - mu_B without cancelling a large constant.  x is clamped to
// [1e-12, 1-1e-12] like clamp_fraction_eps.
template <typename T, typename TC>
PFGB_HD void thermo_mu_off(const TC &c, T xB, T &offA, T &offB) {
    if (c.convex && xB > T(PFGB_XC_CONVEX)) {
        T d = xB - T(PFGB_XC_CONVEX);
        offA = T(c.muA_c) + T(c.dmuA_c) * d + T(c.Kpen_s) * d * d;
        offB = T(c.muB_c) + T(c.dmuB_c) * d + T(c.Kpen_s) * d * d;
        return;
    }
    T x = clamp_eps(xB, T(1e-12));
    T omx = T(1) - x;
    offA = T(c.RT_s) * log(omx) + T(c.L_s) * x * x;
    offB = T(c.RT_s) * log(x) + T(c.L_s) * omx * omx;
}
template <typename T, typename TC>
PFGB_HD void thermo_mu(const TC &c, T xB, T &muA, T &muB) {
    T a, b;
    thermo_mu_off<T>(c, xB, a, b);
    muA = T(c.GA_s) + a;
    muB = T(c.GB_s) + b;
}

// d(mu_B - mu_A)/dx: the reference takes a +-1e-5 central difference of the
// FP64 chemical potentials (thermo_utils.h:552-577).  In FP64 we evaluate the
// same difference quotient; in FP32 the difference would cancel, so the FP32
// path uses the exact derivative of the same functions (the two agree to
// O(1e-10) relative, far below FP32 resolution).
template <typename T> struct GammaEval;
template <> struct GammaEval<double> {
    template <typename TC>
    static PFGB_HD double dmu_diff(const TC &c, double xc) {
        double dx = 1e-5;
        double xp = clamp_eps(xc + dx, 1e-12), xm = clamp_eps(xc - dx, 1e-12);
        double aP, bP, aM, bM;
        thermo_mu<double>(c, xp, aP, bP);
        thermo_mu<double>(c, xm, aM, bM);
        double dA = (aP - aM) / (xp - xm);
        double dB = (bP - bM) / (xp - xm);
        return dB - dA;
    }
};
template <> struct GammaEval<float> {
    template <typename TC>
    static PFGB_HD float dmu_diff(const TC &c, float xc) {
        // d/dx[(G_B - G_A) + RT ln(x/(1-x)) + L((1-x)^2 - x^2)]
        //   = RT / (x (1-x)) - 2 L     (regular-solution branch)
        if (c.convex && xc > float(PFGB_XC_CONVEX)) {
            // both extrapolations are quadratics with equal curvature
            return float(c.ddmu_c);
        }
        float x = clamp_eps(xc, 1e-12f);
        return float(c.RT_s) / (x * (1.0f - x)) - 2.0f * float(c.L_s);
    }
};

template <typename T>
PFGB_HD T c_xB_phi(T xB, T Vm0, T dVm, T Vmc, T h) {
    T den = (Vm0 + dVm * xB) * (T(1) - h) + Vmc * h;
    if (fabs(den) < T(1e-12)) den = (den >= T(0)) ? T(1e-12) : T(-1e-12);
    return T(1) / den;
}

// stabilized_meff, cuda_kernels.cu:30-38
template <typename T>
PFGB_HD T stabilized_meff(T Dm, T g) {
    const T gfloor = T(1.0e-4);
    const T Ds = Dm > T(0) ? Dm : T(0);
    const T gs = (isfinite(g) && g > gfloor) ? g : gfloor;
    const T cap = Ds * T(1000);
    const T v = Ds / gs;
    return (isfinite(v) && v < cap) ? v : cap;
}

// thermodynamic factor, gamma_thermo_nonlinear (thermo_utils.h:552-577)
template <typename T, typename TC>
PFGB_HD T gamma_thermo(const TC &c, T xB, T h, T Vm0, T dVm, T Vmc) {
    T xc = xB;
    if (c.convex && xc > T(0.08)) xc = T(0.08);
    T cb = c_xB_phi(xc, Vm0, dVm, Vmc, h);
    return cb * GammaEval<T>::dmu_diff(c, xc);
}

// numerically stable logistic (sigmoid_from_logit, thermo_utils.h:498-514)
template <typename T>
PFGB_HD T sigmoid_raw(T Y) {
    if (Y >= T(0)) { T e = exp(-Y); return T(1) / (T(1) + e); }
    T e = exp(Y);
    return e / (T(1) + e);
}
template <typename T>
PFGB_HD T sigmoid_clip(T Y, T Yc, T eps) {
    if (Y > Yc) Y = Yc;
    if (Y < -Yc) Y = -Yc;
    T x = sigmoid_raw(Y);
    if (x < eps) x = eps;
    const T hi = one_minus_eps(eps);
    if (x > hi) x = hi;
    return x;
}
template <typename T>
PFGB_HD T logit_clip(T xB, T eps, T Yc) {
    if (xB < eps) xB = eps;
    if (xB > T(1) - eps) xB = T(1) - eps;
    T Y = log(xB / (T(1) - xB));
    if (Y > Yc) return Yc;
    if (Y < -Yc) return -Yc;
    return Y;
}

// ---------------------------------------------------------------------------
// error handling
// ---------------------------------------------------------------------------
#define PFGB_CUDA_TRY(expr)                                                  \
    do {                                                                     \
        cudaError_t e_ = (expr);                                             \
        if (e_ != cudaSuccess) {                                             \
            pfgb_set_error(#expr, e_, __FILE__, __LINE__);                   \
            return PFGB_ERR_CUDA;                                            \
        }                                                                    \
    } while (0)

void pfgb_set_error(const char *what, cudaError_t e, const char *file, int line);
void pfgb_set_error_msg(const char *fmt, ...);
// seeded initial fields (init.cu): phi and xB into device buffers; scratch 2 * 304 doubles
pfgb_status pfgb_seed_fields_device(const pfgb_params *p, double *d_phi, double *d_xB, double *d_scratch,
                                    cudaStream_t stream);
// learned elastic start (fno.cu): device of a model and kernel launches of one forward
int pfgb_fno_device(const pfgb_fno *f);
long long pfgb_fno_forward_launches(const pfgb_fno *f);

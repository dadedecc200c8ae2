// physics.cuh — pointwise physics of the CUDA_STO_PF model, shared by the
// fused pass ops.  T = field precision, TE = elastic precision.
#pragma once

#include "common.cuh"

// Index of Voigt pair (a,b), 0-based, into the 21-vector
// 11 12 13 14 15 16 22 23 24 25 26 33 34 35 36 44 45 46 55 56 66.
__host__ __device__ __forceinline__ int vidx(int a, int b) {
    int lo = a < b ? a : b, hi = a < b ? b : a;
    int start = lo == 0 ? 0 : lo == 1 ? 6 : lo == 2 ? 11 : lo == 3 ? 15 : lo == 4 ? 18 : 20;
    return start + (hi - lo);
}
// tensor (i,j) -> Voigt index 0..5 (xx,yy,zz,yz,xz,xy)
__host__ __device__ __forceinline__ int tvoigt(int i, int j) {
    if (i == j) return i;
    int s = i + j;              // (1,2)->3 yz, (0,2)->2 -> xz, (0,1)->1 -> xy
    return s == 3 ? 3 : (s == 2 ? 4 : 5);
}

// Constants of the physics, FP64 on the host, passed by value to kernels.
// Kernels on FP32 fields take the float copy PhysCT<float> (phys_as): each
// constant is then a plain operand rather than a conversion per use.
template <typename R>
struct PhysCT {
    // grid / time
    R dt, invN;
    // Allen-Cahn phi
    R W, kappa, Lphi;
    R Ldt, gpLdt;      // L_phi dt and L_eta dt, formed in FP64
    // transport
    R Da, Dc;
    R vA, vB, Vm0, dVm, Vmc;
    R mu0, eiv, Yclip, xBeps, hscale;
    R Cdmu;            // mu0 - vA GA_s - vB GB_s - shift (cancellation-free delta_mu)
    R dG;              // GB_s - GA_s
    R shift;
    R e00[6], E0[6];
    R S[21], Sp[21];
    // GP zone
    R gpxB, gpW, gpkap, gpL, gpMGP, gpMb, gpeiso, gpscale;
    R gp_Cg;           // offA(xg)(1-xg) + offB(xg) xg - delta_g0
    int gp, gp_el, act_eta, act_phi;
    int coupling, elastic, zm, prev_level, disable_gamma, xb_raw;
    // GP storage coupling: 0 off; 1 old_rhs (h_alpha floored at haeps in the
    // gamma term); 2 conservative_y_rhs; 3 a storage point update
    int gpy;
    R haeps;           // gp_h_alpha_eps
    // upper cap on the composition seen by the eigenstrain of the elastic
    // solve and the stress (minimize_xB_max_safe once the minimize monitor
    // has clamped xB; above 1 = inactive)
    R xbcap;
    R dx, dy, dz;
    ThermoConstT<R> tc;
};
using PhysC = PhysCT<double>;

template <typename R>
PhysCT<R> phys_as(const PhysC &c) {
    PhysCT<R> o;
    o.dt = R(c.dt); o.invN = R(c.invN);
    o.W = R(c.W); o.kappa = R(c.kappa); o.Lphi = R(c.Lphi);
    o.Ldt = R(c.Lphi * c.dt); o.gpLdt = R(c.gpL * c.dt);
    o.Da = R(c.Da); o.Dc = R(c.Dc);
    o.vA = R(c.vA); o.vB = R(c.vB); o.Vm0 = R(c.Vm0); o.dVm = R(c.dVm); o.Vmc = R(c.Vmc);
    o.mu0 = R(c.mu0); o.eiv = R(c.eiv); o.Yclip = R(c.Yclip); o.xBeps = R(c.xBeps); o.hscale = R(c.hscale);
    o.Cdmu = R(c.Cdmu); o.dG = R(c.dG); o.shift = R(c.shift);
    for (int i = 0; i < 6; ++i) { o.e00[i] = R(c.e00[i]); o.E0[i] = R(c.E0[i]); }
    for (int i = 0; i < 21; ++i) { o.S[i] = R(c.S[i]); o.Sp[i] = R(c.Sp[i]); }
    o.gpxB = R(c.gpxB); o.gpW = R(c.gpW); o.gpkap = R(c.gpkap); o.gpL = R(c.gpL);
    o.gpMGP = R(c.gpMGP); o.gpMb = R(c.gpMb); o.gpeiso = R(c.gpeiso); o.gpscale = R(c.gpscale);
    o.gp_Cg = R(c.gp_Cg);
    o.gp = c.gp; o.gp_el = c.gp_el; o.act_eta = c.act_eta; o.act_phi = c.act_phi;
    o.coupling = c.coupling; o.elastic = c.elastic; o.zm = c.zm; o.prev_level = c.prev_level;
    o.disable_gamma = c.disable_gamma; o.xb_raw = c.xb_raw;
    o.gpy = c.gpy; o.haeps = R(c.haeps);
    o.xbcap = R(c.xbcap); o.dx = R(c.dx); o.dy = R(c.dy); o.dz = R(c.dz);
    o.tc = thermo_as<R>(c.tc);
    return o;
}

// composition entering eps0 on the elastic side: clamp01, then the cap
template <typename T, typename PC>
__device__ __forceinline__ T xB_el(const PC &c, T xB) {
    const T x = clamp01(xB);
    return x < T(c.xbcap) ? x : T(c.xbcap);
}

// Elastic constants in elastic precision (the reference casts S, S_p, eps00,
// E0 to float, main_cuda.cu:28762-28790).
template <typename TE>
struct ElasC {
    TE S[21], Sp[21], e00[6], E0[6];
    TE invN;
};

// xB from the logit Y: clipped form (sigmoid_from_logit) unless the zero mode
// owns the composition, which uses the unclipped logistic
// (apply_pf_Y_zero_mode_shift_kernel, cuda_kernels.cu:3434-3442).
template <typename T, typename PC>
__device__ __forceinline__ T xB_of_Y(const PC &c, T Y) {
    return c.xb_raw ? sigmoid_raw(Y) : sigmoid_clip(Y, T(c.Yclip), T(c.xBeps));
}

// eigenstrain_phi_xB_point / eigenstrain_phi_eta_xB_point
// (cuda_kernels.cu:193-290); gp3 selects the three-phase GP form.
template <typename T, typename TE, typename PC>
__device__ __forceinline__ void eigenstrain(const PC &c, const ElasC<TE> &ec, T phi, T eta,
                                            T xBc, bool gp3, TE e0[6]) {
    if (!gp3) {
        T h = pf_h(phi);
        T epsc = xBc * T(c.eiv);
        T omh = T(1) - h;
#pragma unroll
        for (int a = 0; a < 3; ++a) e0[a] = (TE)(omh * epsc + h * T(ec.e00[a]));
#pragma unroll
        for (int a = 3; a < 6; ++a) e0[a] = (TE)(h * T(ec.e00[a]));
        return;
    }
    T hb = pf_h(phi), he = pf_h(eta);
    T hg = (T(1) - hb) * he, ha = (T(1) - hb) * (T(1) - he);
    T ea = xBc * T(c.eiv);
#pragma unroll
    for (int a = 0; a < 3; ++a) e0[a] = (TE)(ha * ea + hg * T(c.gpeiso) + hb * T(ec.e00[a]));
#pragma unroll
    for (int a = 3; a < 6; ++a) e0[a] = (TE)(hb * T(ec.e00[a]));
}

// Hooke's law with C_eff = C0 + h dC on the elastic strain eps - eps0,
// engineering shear (compute_stress_from_strain_with_effective_stiffness_kernel,
// cuda_kernels.cu:7381-7480).
template <typename T, typename TE, typename PC>
__device__ __forceinline__ void stress_at(const PC &c, const ElasC<TE> &ec, T phi, T eta, T xB,
                                          const TE eps[6], TE sig[6]) {
    TE e0[6];
    eigenstrain<T, TE>(c, ec, phi, eta, xB_el(c, xB), c.gp_el != 0, e0);
    TE el[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) el[a] = eps[a] - e0[a];
    const T h = pf_h(phi);
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        TE acc = 0;
#pragma unroll
        for (int b = 0; b < 6; ++b) {
            const int v = vidx(a, b);
            TE ce = ec.S[v] + (TE)(h * T(ec.Sp[v]));
            acc += (b >= 3 ? TE(2) * ce : ce) * el[b];
        }
        sig[a] = acc;
    }
}

// e^T dC e with engineering shear (compute_Q_voigt, cuda_kernels.cu:162-181)
template <typename T, typename SP>
__device__ __forceinline__ T q_voigt(const SP *Sp, const T el[6]) {
    T e[6] = {el[0], el[1], el[2], T(2) * el[3], T(2) * el[4], T(2) * el[5]};
    T q = 0;
#pragma unroll
    for (int a = 0; a < 6; ++a) {
        q += T(Sp[vidx(a, a)]) * e[a] * e[a];
#pragma unroll
        for (int b = a + 1; b < 6; ++b) q += T(2) * T(Sp[vidx(a, b)]) * e[a] * e[b];
    }
    return q;
}

// explicit Allen-Cahn driving force of phi (compute_phi_rhs_kernel,
// cuda_kernels.cu:390-555): double well + chemical + elastic, with the
// stress given (the reference reads its stored sigma arrays)
template <typename T, typename TE, typename PC>
__device__ __forceinline__ T phi_rhs_sig(const PC &c, const ElasC<TE> &ec, T phi, T eta_raw, T xBraw,
                                         const TE *eps, const TE *sg_) {
    const T hp = pf_hp(phi), gp = pf_gp(phi), h = pf_h(phi);
    const T eta = clamp01(eta_raw);
    const T xB = clamp01(xBraw);
    T f = T(c.W) * gp;
    T offA, offB;
    thermo_mu_off<T>(c.tc, xB, offA, offB);
    const T dmu = T(c.Cdmu) - T(c.vA) * offA - T(c.vB) * offB;
    const T cb = c_xB_phi<T>(xB, T(c.Vm0), T(c.dVm), T(c.Vmc), h);
    const T muA = T(c.tc.GA_s) + offA, muB = T(c.tc.GB_s) + offB;
    const T mt = (T(1) - h) * (muA * (T(1) - xB) + muB * xB) + h * T(c.mu0);
    const T Vma = T(c.Vm0) + T(c.dVm) * xB;
    const T vt = T(c.Vmc) - Vma + T(c.dVm) * (xB - T(c.vB));
    f += cb * hp * (dmu - cb * mt * vt);
    if (c.coupling) {
        T sg[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) sg[a] = T(sg_[a]);
        // eps0 of the two-phase form with float eps00 (as the reference)
        TE e0[6];
        eigenstrain<T, TE>(c, ec, phi, eta, xB, false, e0);
        T el[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) el[a] = T(eps[a]) - T(e0[a]);
        const T Q = q_voigt<T>(c.Sp, el);
        T part;
        const T eps_alpha = xB * T(c.eiv);
        const T diag = -eps_alpha + T(c.eiv) * (xB - T(c.vB));
        if (c.gp_el && c.act_phi) {
            // compute_dgel_dphi_gp_point, cuda_kernels.cu:313-372
            const T he = pf_h(eta);
            T de[6];
#pragma unroll
            for (int a = 0; a < 3; ++a)
                de[a] = hp * (T(c.e00[a]) + (T(1) - he) * diag - he * T(c.gpeiso));
#pragma unroll
            for (int a = 3; a < 6; ++a) de[a] = hp * T(c.e00[a]);
            T dg = -(sg[0] * de[0] + sg[1] * de[1] + sg[2] * de[2] + T(2) * sg[5] * de[5] +
                     T(2) * sg[4] * de[4] + T(2) * sg[3] * de[3]);
            part = T(c.gpscale) * (dg + T(0.5) * hp * Q);
        } else {
            T de[6];
#pragma unroll
            for (int a = 0; a < 3; ++a) de[a] = hp * (T(c.e00[a]) + diag);
#pragma unroll
            for (int a = 3; a < 6; ++a) de[a] = hp * T(c.e00[a]);
            T dg = -(sg[0] * de[0] + sg[1] * de[1] + sg[2] * de[2] + T(2) * sg[5] * de[5] +
                     T(2) * sg[4] * de[4] + T(2) * sg[3] * de[3]);
            part = dg + T(0.5) * hp * Q;
        }
        f += part;
    }
    return f;
}

// phi-only minimize drive (compute_phi_rhs_minimize_kernel,
// cuda_kernels.cu:6298-6374): double well plus, with elasticity on, the
// eigenstrain and stiffness terms of the phi-only eigenstrain h(phi) eps00
// (eigenstrain_phi_only_point, float eps00); no chemistry, no composition.
template <typename T, typename TE, typename PC>
__device__ __forceinline__ T phi_rhs_phi_only(const PC &c, const ElasC<TE> &ec, T phi, const TE *eps,
                                              const TE *sg_) {
    T f = T(c.W) * pf_gp(phi);
    if (c.elastic) {
        const T hp = pf_hp(phi);
        T sg[6], de[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) { sg[a] = T(sg_[a]); de[a] = hp * T(c.e00[a]); }
        const T dg = -(sg[0] * de[0] + sg[1] * de[1] + sg[2] * de[2] +
                       T(2) * (sg[5] * de[5] + sg[4] * de[4] + sg[3] * de[3]));
        TE e0[6];
        eigenstrain<T, TE>(c, ec, phi, T(0), T(0), false, e0);
        T el[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) el[a] = T(eps[a]) - T(e0[a]);
        f += dg + T(0.5) * hp * q_voigt<T>(c.Sp, el);
    }
    return f;
}

// the same with sigma from Hooke's law at (phi, eta, xB): the dynamics step,
// where the stored stress of the reference is that of the current fields
template <typename T, typename TE, typename PC>
__device__ __forceinline__ T phi_rhs(const PC &c, const ElasC<TE> &ec, T phi, T eta_raw, T xBraw,
                                     const TE *eps) {
    TE sg[6];
    if (c.coupling) stress_at<T, TE>(c, ec, phi, eta_raw, xBraw, eps, sg);
    return phi_rhs_sig<T, TE>(c, ec, phi, eta_raw, xBraw, eps, sg);
}

// GP-zone Allen-Cahn driving force of eta (compute_eta_rhs_kernel,
// non-raw-drive branch, cuda_kernels.cu:845-946)
template <typename T, typename TE, typename PC>
__device__ __forceinline__ T eta_rhs(const PC &c, const ElasC<TE> &ec, T eta_raw, T phi_raw,
                                     T xBraw, T sig_hydro) {
    const T eta = clamp01(eta_raw), phi = clamp01(phi_raw);
    const T xa = clamp_eps(xBraw, T(1e-12));
    const T hphi = pf_h(phi), hpe = pf_hp(eta), gpe = pf_gp(eta);
    const T cref = T(1) / (T(c.Vm0) + T(c.dVm) * xa);
    T offA, offB;
    thermo_mu_off<T>(c.tc, xa, offA, offB);
    // g_gp - g_alpha without cancelling the compound constants
    const T dgg = T(c.dG) * (T(c.gpxB) - xa) + T(c.gp_Cg) - (offA * (T(1) - xa) + offB * xa);
    const T d = cref * (T(1) - hphi) * hpe * dgg;
    T el = 0;
    if (c.gp_el && c.act_eta) {
        const T pre = (T(1) - pf_h(phi)) * pf_hp(eta);
        const T ea = clamp01(xa) * T(c.eiv);
        el = T(c.gpscale) * (-sig_hydro * (pre * (T(c.gpeiso) - ea)));
    }
    (void)ec;
    return d + T(c.gpW) * gpe + el;
}

// transport mobility (compute_flux_single_component_kernel :1985 and the
// GP variant :2039)
template <typename T, typename PC>
__device__ __forceinline__ T mobility(const PC &c, T phiY, T etaN, T xBp) {
    if (!c.gp) {
        const T h = pf_h(phiY);
        const T Dm = (T(1) - h) * T(c.Da) + h * T(c.Dc);
        const T G = gamma_thermo<T>(c.tc, xBp, h, T(c.Vm0), T(c.dVm), T(c.Vmc));
        return stabilized_meff<T>(Dm, G);
    }
    const T hb = pf_h(phiY), he = pf_h(etaN);
    const T hg = (T(1) - hb) * he, ha = (T(1) - hb) * (T(1) - he);
    const T Ga = gamma_thermo<T>(c.tc, xBp, T(0), T(c.Vm0), T(c.dVm), T(c.Vmc));
    const T Ma = stabilized_meff<T>(T(c.Da), Ga);
    return ha * Ma + hg * T(c.gpMGP) + hb * T(c.gpMb);
}

/*
 * pf_oracle.c — CPU FP64 restatement of the CUDA_STO_PF dynamics step.
 *
 * TEST INFRASTRUCTURE (the oracle).  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline leg use it; the shipped library never does.
 *
 * Each function cites the reference code it restates.  All arithmetic is
 * FP64; where the reference stores elastic quantities in FP32 (cuda_kernels.cu
 * elastic kernels, main_cuda.cu:28760-28790 casts) the oracle rounds the stored
 * value to float at the same point when elastic_precision == PFGB_PREC_FP32.
 * The step sequence of main_cuda's time loop (main_cuda.cu:28427-31623) is followed literally:
 * one FFT per reference FFT, one dealias per reference dealias call.
 */
#include "pf_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cpx;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* phase functions — phase_functions.h:7-56                             */
/* ------------------------------------------------------------------ */
static inline double o_h(double p) {          /* h = p^3 (6p^2 - 15p + 10) */
    double p2 = p * p, p3 = p2 * p;
    return p3 * (6.0 * p2 - 15.0 * p + 10.0);
}
static inline double o_hp(double p) {         /* h' = 30 p^2 (1-p)^2 */
    double p2 = p * p;
    return 30.0 * p2 * (1.0 - p) * (1.0 - p);
}
static inline double o_g(double p) { return p * p * (1.0 - p) * (1.0 - p); }
static inline double o_gp(double p) {         /* g' = 2p(1-p)(1-2p) */
    return 2.0 * p * (1.0 - p) * (1.0 - 2.0 * p);
}
static inline double o_clamp01(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }
static inline double o_clamp_eps(double v, double eps) {
    return v < eps ? eps : (v > 1.0 - eps ? 1.0 - eps : v);
}

double pfo_h(double p) { return o_h(p); }
double pfo_hp(double p) { return o_hp(p); }
double pfo_gp(double p) { return o_gp(p); }

/* ------------------------------------------------------------------ */
/* thermodynamics — thermo_utils.h:248-579                              */
/* SGTE unary Gibbs energies (Gierlotka 2010 data as used by the        */
/* reference), pseudo-binary regular solution PbTe-Ag2Te.               */
/* ------------------------------------------------------------------ */
#define O_RGAS 8.31446261815324

/* GHSER(T) = a + b T + c T ln T + d T^2 + e T^3 + f / T + g T^-9
 * piecewise in T; one row per (element, range).  thermo_utils.h:280-302 */
typedef struct { double Tmax, a, b, c, d, e, f, g; } sgte_row;
static const sgte_row SGTE_PB[2] = {
    {600.61, -7650.085, 101.700244, -24.5242231, -0.00365895, -2.4395e-7, 0.0, 0.0},
    {1.0e300, -10531.095, 154.243182, -32.4913959, 0.00154613, 0.0, 0.0, 8.05448e25}};
static const sgte_row SGTE_AG[2] = {
    {1234.93, -7209.512, 118.202013, -23.8463314, -0.001790585, -3.98587e-7, -12011.0, 0.0},
    {1.0e300, -15095.252, 190.266404, -33.472, 0.0, 0.0, 0.0, 1.411773e29}};
static const sgte_row SGTE_TE[2] = {
    {722.66, -10544.679, 183.372894, -35.6687, 0.01583435, -5.240417e-6, 155015.0, 0.0},
    {1.0e300, 9160.595, -129.265373, 13.004, -0.0362361, 5.006367e-6, 0.0, -1.28681e30}};

static double sgte_eval(const sgte_row *rows, double T) {
    const sgte_row *r = (T < rows[0].Tmax) ? &rows[0] : &rows[1];
    /* term order follows the reference expression left to right */
    double v = r->a + r->b * T + r->c * T * log(T);
    v += r->d * T * T;
    if (r->e != 0.0) v += r->e * pow(T, 3);
    if (r->f != 0.0) v += r->f / T;
    if (r->g != 0.0) v += r->g * pow(T, -9);
    return v;
}

static double o_G_PbTe(double T) {            /* thermo_utils.h:306-309 */
    return (-76063.2138 + 9.67716633 * T) + sgte_eval(SGTE_PB, T) + sgte_eval(SGTE_TE, T);
}
static double o_G_Ag2Te(double T) {           /* thermo_utils.h:312-316 */
    double per_atom = -10128.93 - 12.645115 * T;
    double g = per_atom + (2.0 / 3.0) * sgte_eval(SGTE_AG, T) + (1.0 / 3.0) * sgte_eval(SGTE_TE, T);
    return 3.0 * g;
}
static double o_Lparam(double T) { return 41212.9 - 18.05 * T; }   /* :325-327 */

#define O_XLIM_CONVEX 0.09                    /* thermo_utils.h:264 */

static double mu_PbTe_cal(double T, double xB) {
    double x = o_clamp_eps(xB, 1e-12);
    return o_G_PbTe(T) + O_RGAS * T * log(1.0 - x) + o_Lparam(T) * x * x;
}
static double mu_Ag2Te_cal(double T, double xB) {
    double x = o_clamp_eps(xB, 1e-12);
    return o_G_Ag2Te(T) + O_RGAS * T * log(x) + o_Lparam(T) * (1.0 - x) * (1.0 - x);
}
static double dmu_PbTe_cal(double T, double xB) {
    double x = o_clamp_eps(xB, 1e-12);
    return -O_RGAS * T / (1.0 - x) + 2.0 * o_Lparam(T) * x;
}
static double dmu_Ag2Te_cal(double T, double xB) {
    double x = o_clamp_eps(xB, 1e-12);
    return O_RGAS * T / x - 2.0 * o_Lparam(T) * (1.0 - x);
}
/* convex extrapolation above X_LIMIT_CONVEX, thermo_utils.h:370-401 */
static double mu_PbTe_raw(double T, double xB, int convex) {
    if (!convex || xB <= O_XLIM_CONVEX) return mu_PbTe_cal(T, xB);
    double xc = O_XLIM_CONVEX, d = xB - xc;
    return mu_PbTe_cal(T, xc) + dmu_PbTe_cal(T, xc) * d + 5000.0 * d * d;
}
static double mu_Ag2Te_raw(double T, double xB, int convex) {
    if (!convex || xB <= O_XLIM_CONVEX) return mu_Ag2Te_cal(T, xB);
    double xc = O_XLIM_CONVEX, d = xB - xc;
    return mu_Ag2Te_cal(T, xc) + dmu_Ag2Te_cal(T, xc) * d + 5000.0 * d * d;
}
static double o_scale(double s) {             /* thermo_utils.h:409-418 */
    return (fabs(s) < 1e-30) ? ((s >= 0.0) ? 1e-30 : -1e-30) : s;
}
static double o_muA(double xB, double T, double s, int cv) { return mu_PbTe_raw(T, xB, cv) / o_scale(s); }
static double o_muB(double xB, double T, double s, int cv) { return mu_Ag2Te_raw(T, xB, cv) / o_scale(s); }

double pfo_mu_A(double xB, double T_K, double scale, int convex) { return o_muA(xB, T_K, scale, convex); }
double pfo_mu_B(double xB, double T_K, double scale, int convex) { return o_muB(xB, T_K, scale, convex); }

/* Newton on RT ln x + L (1-x)^2 = 0, thermo_utils.h:427-452 */
double pfo_xB_eq(double T) {
    double L = o_Lparam(T), RT = O_RGAS * T;
    double x = exp(-L / RT);
    if (x < 1e-9) x = 1e-9;
    if (x > 0.99) x = 0.5;
    for (int it = 0; it < 20; ++it) {
        double f = RT * log(x) + L * (1.0 - x) * (1.0 - x);
        double df = RT / x - 2.0 * L * (1.0 - x);
        double dlt = f / df;
        x -= dlt;
        if (x < 1e-10) x = 1e-10;
        if (x > 0.999) x = 0.999;
        if (fabs(dlt) < 1e-8) break;
    }
    return x;
}

static double o_Vm_alpha(double xB, double Vm0, double dVm) { return Vm0 + dVm * xB; }
static double o_c_xB_phi(double xB, double Vm0, double dVm, double Vmc, double h) {
    double den = o_Vm_alpha(xB, Vm0, dVm) * (1.0 - h) + Vmc * h;   /* :472-479 */
    if (fabs(den) < 1e-12) den = (den >= 0.0) ? 1e-12 : -1e-12;
    return 1.0 / den;
}
static double o_mu_tot_mix(double muA, double muB, double xB, double mu0, double h) {
    double mix = muA * (1.0 - xB) + muB * xB;                      /* :482-486 */
    return (1.0 - h) * mix + h * mu0;
}
static double o_sigmoid(double Y, double Yc, double eps) {       /* :498-514 */
    if (Y > Yc) Y = Yc;
    if (Y < -Yc) Y = -Yc;
    double x;
    if (Y >= 0) { double e = exp(-Y); x = 1.0 / (1.0 + e); }
    else { double e = exp(Y); x = e / (1.0 + e); }
    if (x < eps) x = eps;
    if (x > 1.0 - eps) x = 1.0 - eps;
    return x;
}
static double o_sigmoid_raw(double Y) {     /* pf_zero_mode_sigmoid, cuda_kernels.cu:3391-3399 */
    if (Y >= 0.0) { double e = exp(-Y); return 1.0 / (1.0 + e); }
    double e = exp(Y);
    return e / (1.0 + e);
}
static double o_logit(double xB, double eps, double Yc) {        /* :516-523 */
    if (xB < eps) xB = eps;
    if (xB > 1.0 - eps) xB = 1.0 - eps;
    double Y = log(xB / (1.0 - xB));
    if (Y > Yc) return Yc;
    if (Y < -Yc) return -Yc;
    return Y;
}
double pfo_sigmoid(double Y, double Yc, double eps) { return o_sigmoid(Y, Yc, eps); }
double pfo_logit(double xB, double eps, double Yc) { return o_logit(xB, eps, Yc); }

static double o_Dmix(double h, double Da, double Dc) { return (1.0 - h) * Da + h * Dc; }

/* thermodynamic factor by central difference, thermo_utils.h:552-577 */
static double o_gamma(double xB, double h, double Vm0, double dVm, double Vmc,
                      double T, double s, int cv) {
    double xc = xB;
    if (cv && xc > 0.08) xc = 0.08;
    double cb = o_c_xB_phi(xc, Vm0, dVm, Vmc, h);
    double dx = 1e-5;
    double xp = o_clamp_eps(xc + dx, 1e-12), xm = o_clamp_eps(xc - dx, 1e-12);
    double dA = (o_muA(xp, T, s, cv) - o_muA(xm, T, s, cv)) / (xp - xm);
    double dB = (o_muB(xp, T, s, cv) - o_muB(xm, T, s, cv)) / (xp - xm);
    return cb * (dB - dA);
}
double pfo_gamma(double xB, double h, double Vm0, double dVm, double Vmc,
                 double T_K, double scale, int convex) {
    return o_gamma(xB, h, Vm0, dVm, Vmc, T_K, scale, convex);
}

/* positive bounded mobility, cuda_kernels.cu:30-38 */
static double o_meff(double Dm, double g) {
    const double gfloor = 1.0e-4;
    const double Ds = fmax(Dm, 0.0);
    const double gs = (isfinite(g) && g > gfloor) ? g : gfloor;
    const double cap = Ds * 1000.0;
    const double v = Ds / gs;
    return (isfinite(v) && v < cap) ? v : cap;
}
double pfo_meff(double Dm, double g) { return o_meff(Dm, g); }

void pfo_params_finalize(pfgb_params *p) {   /* main_cuda.cu:15603-15613 */
    double T = p->temperature_C + 273.15;
    if (T < 1.0) T = 1.0;
    p->temperature_K = T;
    double xeq = pfo_xB_eq(T);
    p->xB_eq_matrix = xeq;
    double muA = o_muA(xeq, T, p->mu_reference_scale, p->thermo_convex_extrapolation_enabled);
    double muB = o_muB(xeq, T, p->mu_reference_scale, p->thermo_convex_extrapolation_enabled);
    double vs = p->v_A + p->v_B;
    if (fabs(vs) < 1e-30) vs = (vs >= 0.0) ? 1e-30 : -1e-30;
    p->mu0_compound = (p->v_A * muA + p->v_B * muB) / vs;
}

/* ------------------------------------------------------------------ */
/* state                                                                */
/* ------------------------------------------------------------------ */
struct pfo_state {
    pfgb_params p;
    int Nx, Ny, Nz, NzC;
    size_t N, Nk;
    double invN;
    int fp32e;              /* elastic stored in FP32 like the reference */
    int gp;                 /* model_mode == gp_zone */
    int step;
    /* fields */
    double *phi, *eta, *Y, *xB, *dYdt;
    double *phi_n, *eta_prev, *Y_n, *xB_prev;
    double *xB_gp_old;      /* GP storage coupling: x^n of the feasibility pass */
    double gp_mean_DY;      /* GP storage coupling: <DY> of the step */
    double *rhs, *mu, *scr, *divJ, *lapY, *mass_t, *der_t;
    double *q, *q_before;   /* q_transport_projection_split: matrix storage (1 - h) x */
    int q_rejected, q_redistributed;
    double *cstore;         /* conservative composition modes: C = q + h v_B or q */
    long long cons_limited, cons_constrained;
    cpx *phi_k, *rhs_k, *mu_k, *divJ_k, *Y_k, *scr_k, *eta_k;
    /* elastic */
    double *eps_r[6], *sig_r[6];
    cpx *eps_k[6], *u_k[3], *u_next[3];
    cpx *r_k[3], *d_k[3];   /* increment form: r0 = Phi(u0) - u0 and delta */
    cpx *u_prev[3];         /* extrapolated warm start: u of the step before */
    cpx *u_prev2[3];        /* order 2 and 3: u two steps before */
    cpx *u_prev3[3];        /* order 3 and 4: u three steps before */
    cpx *u_prev4[3];        /* order 4 and 5: u four steps before */
    cpx *u_prev5[3];        /* order 5: u five steps before */
    cpx *dm_k[3];           /* Chebyshev semi-iteration: the iterate before delta */
    int cheb;               /* elastic_chebyshev with the increment form */
    double cheb_gam, cheb_sig;
    int warm_count;         /* solutions available for the warm start */
    int warm_valid;
    /* k tables */
    double *kx, *ky, *kz;
    unsigned char *mx, *my, *mz;  /* 1 = dealiased (zeroed) */
    double target_mass;
    /* minimize */
    double *mlap, *mg;
    double lambda_vol, V0_target, prev_F_total;
    int min_iter, conv_count, converged_iter;
};

static inline double rf(const pfo_state *s, double v) { return s->fp32e ? (double)(float)v : v; }

/* kx_wrap / ky_wrap / kz_wrap, cuda_common.h:68-82 */
static double kwrap(int i, int n, double d) {
    int ii = (i <= n / 2) ? i : i - n;
    return 2.0 * M_PI * ii / (d * n);
}
/* 2/3-rule predicate, cuda_kernels.cu:103-131 */
static int dealias_cut(double k, double d) {
    const double kmax = M_PI * (2.0 / 3.0) / d;
    return fabs(k) >= kmax;
}

static void *xalloc(size_t n) {
    void *p = calloc(n ? n : 1, 1);
    return p;
}

pfo_state *pfo_create(const pfgb_params *pin) {
    pfo_state *s = (pfo_state *)xalloc(sizeof(pfo_state));
    s->p = *pin;
    pfo_params_finalize(&s->p);
    s->Nx = pin->Nx; s->Ny = pin->Ny; s->Nz = pin->Nz; s->NzC = pin->Nz / 2 + 1;
    s->N = (size_t)s->Nx * s->Ny * s->Nz;
    s->Nk = (size_t)s->Nx * s->Ny * s->NzC;
    s->invN = 1.0 / (double)s->N;
    s->fp32e = (pin->elastic_precision == PFGB_PREC_FP32);
    s->gp = (pin->model_mode == PFGB_MODEL_GP_ZONE);
    const size_t rb = sizeof(double) * s->N, kb = sizeof(cpx) * s->Nk;
    double **rf_[] = {&s->phi, &s->eta, &s->Y, &s->xB, &s->dYdt, &s->phi_n, &s->eta_prev,
                      &s->Y_n, &s->xB_prev, &s->rhs, &s->mu, &s->scr, &s->divJ, &s->lapY,
                      &s->mass_t, &s->der_t, &s->q, &s->q_before, &s->cstore, &s->xB_gp_old};
    for (size_t i = 0; i < sizeof(rf_) / sizeof(rf_[0]); ++i) *rf_[i] = (double *)xalloc(rb);
    cpx **kf_[] = {&s->phi_k, &s->rhs_k, &s->mu_k, &s->divJ_k, &s->Y_k, &s->scr_k, &s->eta_k};
    for (size_t i = 0; i < sizeof(kf_) / sizeof(kf_[0]); ++i) *kf_[i] = (cpx *)xalloc(kb);
    for (int c = 0; c < 6; ++c) {
        s->eps_r[c] = (double *)xalloc(rb);
        s->sig_r[c] = (double *)xalloc(rb);
        s->eps_k[c] = (cpx *)xalloc(kb);
    }
    for (int c = 0; c < 3; ++c) {
        s->u_k[c] = (cpx *)xalloc(kb);
        s->u_next[c] = (cpx *)xalloc(kb);
        s->r_k[c] = (cpx *)xalloc(kb);
        s->d_k[c] = (cpx *)xalloc(kb);
        s->u_prev[c] = (cpx *)xalloc(kb);
        s->u_prev2[c] = (cpx *)xalloc(kb);
        s->u_prev3[c] = (cpx *)xalloc(kb);
        s->u_prev4[c] = (cpx *)xalloc(kb);
        s->u_prev5[c] = (cpx *)xalloc(kb);
        s->dm_k[c] = (cpx *)xalloc(kb);
    }
    if (pin->elastic_chebyshev && pin->elastic_increment_form) {
        double a, b;
        if (pfo_chebyshev_bounds(pin->S, pin->S_p, &a, &b)) {
            s->cheb = 1;
            s->cheb_gam = 2.0 / (2.0 - a - b);
            s->cheb_sig = (b - a) / (2.0 - a - b);
        }
    }
    s->mlap = (double *)xalloc(rb);
    s->mg = (double *)xalloc(rb);
    s->V0_target = pin->minimize_V0;
    s->prev_F_total = NAN;
    if (pin->mode == PFGB_MODE_MINIMIZE) s->p.dt = pin->minimize_dt;   /* main_cuda.cu:24432-24435 */
    s->kx = (double *)xalloc(sizeof(double) * s->Nx);
    s->ky = (double *)xalloc(sizeof(double) * s->Ny);
    s->kz = (double *)xalloc(sizeof(double) * s->NzC);
    s->mx = (unsigned char *)xalloc(s->Nx);
    s->my = (unsigned char *)xalloc(s->Ny);
    s->mz = (unsigned char *)xalloc(s->NzC);
    for (int i = 0; i < s->Nx; ++i) { s->kx[i] = kwrap(i, s->Nx, pin->dx); s->mx[i] = dealias_cut(s->kx[i], pin->dx); }
    for (int j = 0; j < s->Ny; ++j) { s->ky[j] = kwrap(j, s->Ny, pin->dy); s->my[j] = dealias_cut(s->ky[j], pin->dy); }
    for (int k = 0; k < s->NzC; ++k) {
        s->kz[k] = 2.0 * M_PI * k / (pin->dz * s->Nz);
        s->mz[k] = dealias_cut(s->kz[k], pin->dz);
    }
    return s;
}

void pfo_destroy(pfo_state *s) {
    if (!s) return;
    double *rr[] = {s->phi, s->eta, s->Y, s->xB, s->dYdt, s->phi_n, s->eta_prev, s->Y_n,
                    s->xB_prev, s->rhs, s->mu, s->scr, s->divJ, s->lapY, s->mass_t, s->der_t, s->q,
                    s->q_before, s->cstore, s->xB_gp_old};
    for (size_t i = 0; i < sizeof(rr) / sizeof(rr[0]); ++i) free(rr[i]);
    cpx *kk[] = {s->phi_k, s->rhs_k, s->mu_k, s->divJ_k, s->Y_k, s->scr_k, s->eta_k};
    for (size_t i = 0; i < sizeof(kk) / sizeof(kk[0]); ++i) free(kk[i]);
    for (int c = 0; c < 6; ++c) { free(s->eps_r[c]); free(s->sig_r[c]); free(s->eps_k[c]); }
    for (int c = 0; c < 3; ++c) {
        free(s->u_k[c]); free(s->u_next[c]); free(s->r_k[c]); free(s->d_k[c]); free(s->u_prev[c]); free(s->u_prev2[c]); free(s->u_prev3[c]); free(s->u_prev4[c]); free(s->u_prev5[c]); free(s->dm_k[c]);
    }
    free(s->kx); free(s->ky); free(s->kz); free(s->mx); free(s->my); free(s->mz);
    free(s->mlap); free(s->mg);
    free(s);
}

int pfo_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* deterministic sum: fixed 4096-element blocks, block partials summed in order */
static double dsum(const double *a, size_t n) {
    const size_t B = 4096;
    size_t nb = (n + B - 1) / B;
    double *part = (double *)malloc(sizeof(double) * (nb ? nb : 1));
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < (long long)nb; ++b) {
        size_t lo = (size_t)b * B, hi = lo + B < n ? lo + B : n;
        double acc = 0.0;
        for (size_t i = lo; i < hi; ++i) acc += a[i];
        part[b] = acc;
    }
    double t = 0.0;
    for (size_t b = 0; b < nb; ++b) t += part[b];
    free(part);
    return t;
}

/* 3D transforms on the state's grid */
static void fwd(pfo_state *s, const double *r, cpx *k) {
    pfo_fft3d_r2c(s->Nx, s->Ny, s->Nz, r, (double *)k);
}
static void inv(pfo_state *s, const cpx *k, double *r) {
    pfo_fft3d_c2r(s->Nx, s->Ny, s->Nz, (const double *)k, r);
}

#define KLOOP_BEGIN(s)                                                        \
    _Pragma("omp parallel for schedule(static)")                              \
    for (long long idx_ = 0; idx_ < (long long)(s)->Nk; ++idx_) {            \
        const size_t idx = (size_t)idx_;                                      \
        const int kk_ = (int)(idx % (s)->NzC);                                \
        const int jj_ = (int)((idx / (s)->NzC) % (s)->Ny);                    \
        const int ii_ = (int)(idx / ((size_t)(s)->NzC * (s)->Ny));            \
        (void)kk_; (void)jj_; (void)ii_;
#define KLOOP_END }

#define RLOOP_BEGIN(s)                                                        \
    _Pragma("omp parallel for schedule(static)")                              \
    for (long long idx_ = 0; idx_ < (long long)(s)->N; ++idx_) {             \
        const size_t idx = (size_t)idx_;
#define RLOOP_END }

static inline int masked(const pfo_state *s, int i, int j, int k) {
    return s->mx[i] | s->my[j] | s->mz[k];
}

/* dealias_23_kernel, cuda_kernels.cu:103-131 (+ the float variant :135-160) */
static void dealias(pfo_state *s, cpx *f) {
    KLOOP_BEGIN(s)
        if (masked(s, ii_, jj_, kk_)) { f[idx].re = 0.0; f[idx].im = 0.0; }
    KLOOP_END
}

static double k2_at(const pfo_state *s, int i, int j, int k) {
    /* kspace_build_kernel, cuda_common.cu:51-73 */
    double kx = s->kx[i], ky = s->ky[j], kz = s->kz[k];
    return kx * kx + ky * ky + kz * kz;
}

/* ------------------------------------------------------------------ */
/* elastic solve — main_cuda.cu:28760-29160                             */
/* ------------------------------------------------------------------ */
typedef struct {
    double S[21], Sp[21], e00[6], E0[6];
} elast_consts;

/* indices into the 21-vector: 11 12 13 14 15 16 22 23 24 25 26 33 34 35 36 44 45 46 55 56 66 */
enum { C11, C12, C13, C14, C15, C16, C22, C23, C24, C25, C26, C33, C34, C35, C36,
       C44, C45, C46, C55, C56, C66 };

/* symmetric 6x6 accessor (1-based Voigt a,b) */
static double voigt(const double *c21, int a, int b) {
    static const int map[7][7] = {
        {0, 0, 0, 0, 0, 0, 0},
        {0, C11, C12, C13, C14, C15, C16},
        {0, C12, C22, C23, C24, C25, C26},
        {0, C13, C23, C33, C34, C35, C36},
        {0, C14, C24, C34, C44, C45, C46},
        {0, C15, C25, C35, C45, C55, C56},
        {0, C16, C26, C36, C46, C56, C66}};
    return c21[map[a][b]];
}

/* Voigt engineering vector from tensor strain xx,yy,zz,yz,xz,xy */
static void eng(const double *e, double *v) {
    v[0] = e[0]; v[1] = e[1]; v[2] = e[2];
    v[3] = 2.0 * e[3]; v[4] = 2.0 * e[4]; v[5] = 2.0 * e[5];
}

/* eigenstrain_phi_xB_point / eigenstrain_phi_eta_xB_point,
 * cuda_kernels.cu:193-290 */
static void eigen_point(const pfo_state *s, const elast_consts *ec, double phi, double eta,
                        double xB_clamped, int gp_elastic, double *e0) {
    const pfgb_params *P = &s->p;
    if (!gp_elastic) {
        double h = o_h(phi);
        double epsc = xB_clamped * P->eps_iso_over_vB;
        double omh = 1.0 - h;
        for (int c = 0; c < 3; ++c) e0[c] = rf(s, omh * epsc + h * ec->e00[c]);
        for (int c = 3; c < 6; ++c) e0[c] = rf(s, h * ec->e00[c]);
        return;
    }
    double hb = o_h(phi), he = o_h(eta);
    double hg = (1.0 - hb) * he, ha = (1.0 - hb) * (1.0 - he);
    double ea = xB_clamped * P->eps_iso_over_vB;
    for (int c = 0; c < 3; ++c) e0[c] = rf(s, ha * ea + hg * P->gp_eps_iso + hb * ec->e00[c]);
    for (int c = 3; c < 6; ++c) e0[c] = rf(s, hb * ec->e00[c]);
}

/* acoustic tensor K_ij = k_a C_iajb k_b (the "g" combinations of
 * cuda_kernels.cu:6538-6567 / K of :6822-6866) */
static void acoustic(const double *S, double kx, double ky, double kz, double K[3][3]) {
    const double kv[3] = {kx, ky, kz};
    /* Voigt index of (i,j) */
    static const int vi[3][3] = {{1, 6, 5}, {6, 2, 4}, {5, 4, 3}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    acc += kv[a] * voigt(S, vi[i][a], vi[j][b]) * kv[b];
            K[i][j] = acc;
        }
}

static int inverse3(double K[3][3], double G[3][3]) {
    double det = K[0][0] * (K[1][1] * K[2][2] - K[1][2] * K[2][1])
               - K[0][1] * (K[1][0] * K[2][2] - K[1][2] * K[2][0])
               + K[0][2] * (K[1][0] * K[2][1] - K[1][1] * K[2][0]);
    if (fabs(det) < 1e-30) return 0;
    G[0][0] = (K[1][1] * K[2][2] - K[1][2] * K[2][1]) / det;
    G[0][1] = (K[0][2] * K[2][1] - K[0][1] * K[2][2]) / det;
    G[0][2] = (K[0][1] * K[1][2] - K[0][2] * K[1][1]) / det;
    G[1][0] = (K[1][2] * K[2][0] - K[1][0] * K[2][2]) / det;
    G[1][1] = (K[0][0] * K[2][2] - K[0][2] * K[2][0]) / det;
    G[1][2] = (K[0][2] * K[1][0] - K[0][0] * K[1][2]) / det;
    G[2][0] = (K[1][0] * K[2][1] - K[1][1] * K[2][0]) / det;
    G[2][1] = (K[0][1] * K[2][0] - K[0][0] * K[2][1]) / det;
    G[2][2] = (K[0][0] * K[1][1] - K[0][1] * K[1][0]) / det;
    return 1;
}

/* u_k = -i G(k) (k . tau_k) for a symmetric source tau (6 components):
 * compute_displacement_from_eigenstrain_k_kernel (tau = C0:eps0,
 * :6734-6998) and compute_displacement_from_hij_green_kernel (tau = h,
 * :6484-6634); k = 0 -> 0, |det| < 1e-30 -> 0. */
static void green_apply(pfo_state *s, const elast_consts *ec, cpx **tau_k, int tau_is_eigen,
                        cpx **u_out) {
    static const int vi[3][3] = {{1, 6, 5}, {6, 2, 4}, {5, 4, 3}};
    static const int comp_of[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}}; /* xx yy zz yz xz xy */
    KLOOP_BEGIN(s)
        double kx = s->kx[ii_], ky = s->ky[jj_], kz = s->kz[kk_];
        if (ii_ == 0 && jj_ == 0 && kk_ == 0) {
            for (int c = 0; c < 3; ++c) { u_out[c][idx].re = 0.0; u_out[c][idx].im = 0.0; }
            continue;
        }
        double K[3][3], G[3][3];
        acoustic(ec->S, kx, ky, kz, K);
        if (!inverse3(K, G)) {
            for (int c = 0; c < 3; ++c) { u_out[c][idx].re = 0.0; u_out[c][idx].im = 0.0; }
            continue;
        }
        const double kv[3] = {kx, ky, kz};
        /* t_i = k_j tau_ij ; for the eigen source tau_ij = C_ijkl eps0_kl */
        double tr[3] = {0, 0, 0}, ti[3] = {0, 0, 0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                double ar, ai;
                if (tau_is_eigen) {
                    ar = 0.0; ai = 0.0;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) {
                            double c = voigt(ec->S, vi[i][j], vi[a][b]);
                            const cpx e = tau_k[comp_of[a][b]][idx];
                            ar += c * e.re; ai += c * e.im;
                        }
                } else {
                    const cpx e = tau_k[comp_of[i][j]][idx];
                    ar = e.re; ai = e.im;
                }
                tr[i] += kv[j] * ar; ti[i] += kv[j] * ai;
            }
        for (int c = 0; c < 3; ++c) {
            double sr = 0.0, si = 0.0;
            for (int d = 0; d < 3; ++d) { sr += G[c][d] * tr[d]; si += G[c][d] * ti[d]; }
            /* u = -i (sr + i si) = si - i sr */
            u_out[c][idx].re = rf(s, si);
            u_out[c][idx].im = rf(s, -sr);
        }
    KLOOP_END
}

/* compute_strain_from_displacement_k_kernel, cuda_kernels.cu:6673-6730 */
static void strain_from_u(pfo_state *s, cpx **u, cpx **e) {
    KLOOP_BEGIN(s)
        double kv[3] = {rf(s, s->kx[ii_]), rf(s, s->ky[jj_]), rf(s, s->kz[kk_])};
        const cpx uu[3] = {u[0][idx], u[1][idx], u[2][idx]};
        /* eps_ij = i (k_i u_j + k_j u_i) / 2 */
        static const int pr[6][2] = {{0, 0}, {1, 1}, {2, 2}, {1, 2}, {0, 2}, {0, 1}};
        for (int c = 0; c < 6; ++c) {
            int a = pr[c][0], b = pr[c][1];
            double tr_, ti_;
            if (a == b) { tr_ = kv[a] * uu[a].re; ti_ = kv[a] * uu[a].im; }
            else {
                tr_ = 0.5 * (kv[a] * uu[b].re + kv[b] * uu[a].re);
                ti_ = 0.5 * (kv[a] * uu[b].im + kv[b] * uu[a].im);
            }
            e[c][idx].re = rf(s, -ti_);
            e[c][idx].im = rf(s, tr_);
        }
    KLOOP_END
}

static void elastic_fwd(pfo_state *s, double *r, cpx *k) {
    fwd(s, r, k);
    if (s->fp32e) {
        for (size_t i = 0; i < s->Nk; ++i) { k[i].re = (double)(float)k[i].re; k[i].im = (double)(float)k[i].im; }
    }
}
static void elastic_inv(pfo_state *s, const cpx *k, double *r) {
    inv(s, k, r);
    if (s->fp32e) for (size_t i = 0; i < s->N; ++i) r[i] = (double)(float)r[i];
}

/* the elastic constants in elastic precision (the reference casts S, S_p,
 * eps00 and E0 to float, main_cuda.cu:28762-28790) */
static void elastic_consts(pfo_state *s, elast_consts *ec) {
    const pfgb_params *P = &s->p;
    for (int c = 0; c < 21; ++c) { ec->S[c] = rf(s, P->S[c]); ec->Sp[c] = rf(s, P->S_p[c]); }
    for (int c = 0; c < 6; ++c) { ec->e00[c] = rf(s, P->eps00[c]); ec->E0[c] = rf(s, P->E0[c]); }
}

/* compute_strain_with_perturbation_kernel, cuda_kernels.cu:7002-7157:
 * h = C0:eps - (C0 + h dC):(eps + E0 - eps0) over s->eps_r in place (the
 * increment form's linear part: eps only) */
static void polarization(pfo_state *s, const elast_consts *ecp, int gp_el, int lin) {
    const elast_consts ec = *ecp;
    RLOOP_BEGIN(s)
        double e[6], e0[6];
        for (int c = 0; c < 6; ++c) e[c] = s->eps_r[c][idx];
        eigen_point(s, &ec, s->phi[idx], s->eta[idx], o_clamp01(s->xB[idx]), gp_el, e0);
        double hw = o_h(s->phi[idx]);   /* stiffness_beta_weight_point */
        double ev[6], tv[6];
        double tot[6];
        for (int c = 0; c < 6; ++c) tot[c] = lin ? e[c] : e[c] + ec.E0[c] - e0[c];
        eng(e, ev); eng(tot, tv);
        static const int rowv[6] = {1, 2, 3, 4, 5, 6};
        for (int c = 0; c < 6; ++c) {
            double acc = 0.0;
            for (int b = 0; b < 6; ++b) {
                double c0 = voigt(ec.S, rowv[c], b + 1);
                double ce = c0 + rf(s, hw * voigt(ec.Sp, rowv[c], b + 1));
                acc += c0 * ev[b] - ce * tv[b];
            }
            s->eps_r[c][idx] = rf(s, acc);
        }
    RLOOP_END
}

/* test hooks for the pinning tests: the polarization on given strains
 * (eps: 6 N, Voigt xx yy zz yz xz xy, tensor strain) and the Green's
 * contraction of given polarization spectra (tau: 6 Nk, u: 3 Nk complex) */
void pfo_test_polarization(pfo_state *s, int lin, const double *phi, const double *eta, const double *xB,
                           const double *eps, double *out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->phi, phi, b);
    memcpy(s->eta, eta, b);
    memcpy(s->xB, xB, b);
    for (int c = 0; c < 6; ++c) memcpy(s->eps_r[c], eps + (size_t)c * s->N, b);
    elast_consts ec;
    elastic_consts(s, &ec);
    polarization(s, &ec, s->gp && s->p.gp_elastic_enabled, lin);
    for (int c = 0; c < 6; ++c) memcpy(out + (size_t)c * s->N, s->eps_r[c], b);
}
void pfo_test_green(pfo_state *s, const double *tau, double *u) {
    const size_t kb = sizeof(cpx) * s->Nk;
    for (int c = 0; c < 6; ++c) memcpy(s->eps_k[c], tau + 2 * (size_t)c * s->Nk, kb);
    elast_consts ec;
    elastic_consts(s, &ec);
    green_apply(s, &ec, s->eps_k, 0, s->u_next);
    for (int c = 0; c < 3; ++c) memcpy(u + 2 * (size_t)c * s->Nk, s->u_next[c], kb);
}

static int elastic_solve(pfo_state *s, pfgb_step_stats *st) {
    const pfgb_params *P = &s->p;
    elast_consts ec;
    elastic_consts(s, &ec);
    const double invNf = rf(s, s->invN);
    const int gp_el = s->gp && P->gp_elastic_enabled;
    const int accel = P->elastic_enabled && (P->elastic_warm_start_enabled || P->elastic_residual_control_enabled);
    const int warm_used = accel && s->warm_valid;

    if (!warm_used) {
        /* eigenstrain -> R2C -> homogeneous displacement (:28813-28868) */
        RLOOP_BEGIN(s)
            double e0[6];
            eigen_point(s, &ec, s->phi[idx], s->eta[idx], o_clamp01(s->xB[idx]), gp_el, e0);
            for (int c = 0; c < 6; ++c) s->eps_r[c][idx] = e0[c];
        RLOOP_END
        for (int c = 0; c < 6; ++c) { elastic_fwd(s, s->eps_r[c], s->eps_k[c]); dealias(s, s->eps_k[c]); }
        green_apply(s, &ec, s->eps_k, 1, s->u_k);
        for (int c = 0; c < 3; ++c) dealias(s, s->u_k[c]);
    }

    if (warm_used && P->elastic_warm_start_extrapolate) {
        /* u0 the polynomial extrapolation through the last m + 1 solutions,
         * m = min(elastic_warm_start_extrapolate, solutions - 1):
         * 2 u^n - u^{n-1}; 3 u^n - 3 u^{n-1} + u^{n-2};
         * 4 u^n - 6 u^{n-1} + 4 u^{n-2} - u^{n-3};
         * 5 u^n - 10 u^{n-1} + 10 u^{n-2} - 5 u^{n-3} + u^{n-4};
         * 6, -15, 20, -15, 6, -1; the history shifts by one */
        int m = P->elastic_warm_start_extrapolate;
        if (m > s->warm_count - 1) m = s->warm_count - 1;
        static const double cf[6][6] = {{1, 0, 0, 0, 0, 0}, {2, -1, 0, 0, 0, 0}, {3, -3, 1, 0, 0, 0},
                                        {4, -6, 4, -1, 0, 0}, {5, -10, 10, -5, 1, 0}, {6, -15, 20, -15, 6, -1}};
        const double *w = cf[m < 0 ? 0 : m];
        KLOOP_BEGIN(s)
            for (int c = 0; c < 3; ++c) {
                const cpx h0 = s->u_k[c][idx], h1 = s->u_prev[c][idx], h2 = s->u_prev2[c][idx],
                          h3 = s->u_prev3[c][idx], h4 = s->u_prev4[c][idx], h5 = s->u_prev5[c][idx];
                if (m >= 1) {
                    double re = w[0] * h0.re + w[1] * h1.re, im = w[0] * h0.im + w[1] * h1.im;
                    if (m >= 2) { re += w[2] * h2.re; im += w[2] * h2.im; }
                    if (m >= 3) { re += w[3] * h3.re; im += w[3] * h3.im; }
                    if (m >= 4) { re += w[4] * h4.re; im += w[4] * h4.im; }
                    if (m >= 5) { re += w[5] * h5.re; im += w[5] * h5.im; }
                    s->u_k[c][idx].re = rf(s, re);
                    s->u_k[c][idx].im = rf(s, im);
                }
                s->u_prev5[c][idx] = h4;
                s->u_prev4[c][idx] = h3;
                s->u_prev3[c][idx] = h2;
                s->u_prev2[c][idx] = h1;
                s->u_prev[c][idx] = h0;
            }
        KLOOP_END
    }
    int iter = accel ? 0 : 1;
    int conv = accel ? 0 : 1;
    double rel = NAN;
    /* increment form (elastic_increment_form): the first update is the full
     * u1 = Phi(u0); then delta <- r0 + L delta with r0 = u1 - u0 and L the
     * linear part h_lin = -(h dC):eps(delta) of the operator */
    const int inc = accel && P->elastic_increment_form;
    /* Chebyshev semi-iteration of the increment (elastic_chebyshev):
     * y = delta + gam (g - delta), delta_new = delta_prev + rho (y - delta_prev),
     * rho_2 = 2 / (2 - sig^2), rho_{k+1} = 1 / (1 - sig^2 rho_k / 4); the first
     * update is delta_1 = gam r0 from delta_0 = 0 */
    const int chb = inc && s->cheb;
    int cheb_it = 0;
    double rho = 1.0;
    for (;;) {
        const int lin = inc && iter >= 1;
        strain_from_u(s, lin ? s->d_k : s->u_k, s->eps_k);
        for (int c = 0; c < 6; ++c) dealias(s, s->eps_k[c]);
        for (int c = 0; c < 6; ++c) elastic_inv(s, s->eps_k[c], s->eps_r[c]);
        /* normalize_strain_kernel (float invN) */
        for (int c = 0; c < 6; ++c) {
            double *e = s->eps_r[c];
            RLOOP_BEGIN(s) e[idx] = rf(s, e[idx] * invNf); RLOOP_END
        }
        polarization(s, &ec, gp_el, lin);
        for (int c = 0; c < 6; ++c) { elastic_fwd(s, s->eps_r[c], s->eps_k[c]); dealias(s, s->eps_k[c]); }
        cpx **target = accel ? s->u_next : s->u_k;
        green_apply(s, &ec, s->eps_k, 0, target);
        for (int c = 0; c < 3; ++c) dealias(s, target[c]);
        if (inc) {
            /* the same residual on the increment iterates */
            double *dif = s->mass_t, *ref = s->der_t;
            if (chb && lin) {
                const double s2 = s->cheb_sig * s->cheb_sig;
                rho = cheb_it == 0 ? 2.0 / (2.0 - s2) : 1.0 / (1.0 - 0.25 * s2 * rho);
                ++cheb_it;
            }
            KLOOP_BEGIN(s)
                double w = (kk_ == 0 || ((s->Nz % 2) == 0 && kk_ == s->Nz / 2)) ? 1.0 : 2.0;
                double ld = 0.0, lr = 0.0;
                for (int c = 0; c < 3; ++c) {
                    const cpx v = s->u_next[c][idx];
                    if (!lin) {   /* r0 = u1 - u0, delta = r0, u_new = u1 */
                        cpx r = {rf(s, v.re - s->u_k[c][idx].re), rf(s, v.im - s->u_k[c][idx].im)};
                        s->r_k[c][idx] = r;
                        if (chb) {
                            const cpx x1 = {rf(s, s->cheb_gam * r.re), rf(s, s->cheb_gam * r.im)};
                            const cpx z = {0.0, 0.0};
                            s->d_k[c][idx] = x1;
                            s->dm_k[c][idx] = z;
                        } else {
                            s->d_k[c][idx] = r;
                        }
                        ld += r.re * r.re + r.im * r.im;
                        lr += v.re * v.re + v.im * v.im;
                    } else {      /* delta_new = r0 + L delta, u_new = u0 + delta_new */
                        cpx dn = {rf(s, s->r_k[c][idx].re + v.re), rf(s, s->r_k[c][idx].im + v.im)};
                        const cpx d = s->d_k[c][idx];
                        const double dr = dn.re - d.re, di = dn.im - d.im;
                        const double ur = rf(s, s->u_k[c][idx].re + dn.re), ui = rf(s, s->u_k[c][idx].im + dn.im);
                        if (chb) {
                            const cpx xm = s->dm_k[c][idx];
                            const double yr = d.re + s->cheb_gam * dr, yi = d.im + s->cheb_gam * di;
                            const cpx xn = {rf(s, xm.re + rho * (yr - xm.re)), rf(s, xm.im + rho * (yi - xm.im))};
                            s->dm_k[c][idx] = d;
                            s->d_k[c][idx] = xn;
                        } else {
                            s->d_k[c][idx] = dn;
                        }
                        ld += dr * dr + di * di;
                        lr += ur * ur + ui * ui;
                    }
                }
                dif[idx] = w * ld; ref[idx] = w * lr;
            KLOOP_END
            double ds = dsum(dif, s->Nk), rs = dsum(ref, s->Nk);
            if (!isfinite(ds) || !isfinite(rs) || ds < 0.0 || rs < 0.0) return PFGB_ERR_NONFINITE;
            rel = sqrt(ds / fmax(rs, P->elastic_residual_absolute_floor));
            ++iter;
            if (iter >= P->elastic_iter_min && rel <= P->elastic_residual_tolerance) { conv = 1; break; }
            if (iter >= P->elastic_iter_max) break;
        } else if (accel) {
            /* compute_elastic_displacement_residual_kernel, :6436-6467 */
            double *dif = s->mass_t, *ref = s->der_t;
            /* residual arrays sized Nk <= N */
            KLOOP_BEGIN(s)
                double w = (kk_ == 0 || ((s->Nz % 2) == 0 && kk_ == s->Nz / 2)) ? 1.0 : 2.0;
                double ld = 0.0, lr = 0.0;
                for (int c = 0; c < 3; ++c) {
                    double dr = s->u_next[c][idx].re - s->u_k[c][idx].re;
                    double di = s->u_next[c][idx].im - s->u_k[c][idx].im;
                    double nr = s->u_next[c][idx].re, ni = s->u_next[c][idx].im;
                    ld += dr * dr + di * di;
                    lr += nr * nr + ni * ni;
                }
                dif[idx] = w * ld; ref[idx] = w * lr;
            KLOOP_END
            double ds = dsum(dif, s->Nk), rs = dsum(ref, s->Nk);
            if (!isfinite(ds) || !isfinite(rs) || ds < 0.0 || rs < 0.0) return PFGB_ERR_NONFINITE;
            rel = sqrt(ds / fmax(rs, P->elastic_residual_absolute_floor));
            for (int c = 0; c < 3; ++c) { cpx *t = s->u_k[c]; s->u_k[c] = s->u_next[c]; s->u_next[c] = t; }
            ++iter;
            if (iter >= P->elastic_iter_min && rel <= P->elastic_residual_tolerance) { conv = 1; break; }
            if (iter >= P->elastic_iter_max) break;
        } else {
            ++iter;
            if (iter >= P->elastic_iter_max) break;
        }
    }
    if (inc) {
        KLOOP_BEGIN(s)
            for (int c = 0; c < 3; ++c) {
                s->u_k[c][idx].re = rf(s, s->u_k[c][idx].re + s->d_k[c][idx].re);
                s->u_k[c][idx].im = rf(s, s->u_k[c][idx].im + s->d_k[c][idx].im);
            }
        KLOOP_END
    }
    if (accel) { s->warm_valid = 1; s->warm_count++; }
    if (st) {
        st->elastic_iterations = iter;
        st->elastic_converged = conv;
        st->elastic_warm_start_used = warm_used;
        st->elastic_relative_residual = rel;
        st->elastic_iterations_total += iter;
    }
    if (accel && !conv && P->elastic_fail_on_nonconvergence) return PFGB_ERR_NONCONVERGED;

    /* finalize (:29104-29160): strain from u, C2R, normalize, +E0, stress */
    strain_from_u(s, s->u_k, s->eps_k);
    for (int c = 0; c < 6; ++c) dealias(s, s->eps_k[c]);
    for (int c = 0; c < 6; ++c) elastic_inv(s, s->eps_k[c], s->eps_r[c]);
    for (int c = 0; c < 6; ++c) {
        double *e = s->eps_r[c];
        const double E0c = ec.E0[c];
        RLOOP_BEGIN(s) e[idx] = rf(s, rf(s, e[idx] * invNf) + E0c); RLOOP_END
    }
    /* compute_stress_from_strain_with_effective_stiffness_kernel, :7381-7480 */
    RLOOP_BEGIN(s)
        double e0[6], el[6], ev[6];
        eigen_point(s, &ec, s->phi[idx], s->eta[idx], o_clamp01(s->xB[idx]), gp_el, e0);
        for (int c = 0; c < 6; ++c) el[c] = rf(s, s->eps_r[c][idx] - e0[c]);
        eng(el, ev);
        double hw = o_h(s->phi[idx]);
        for (int c = 0; c < 6; ++c) {
            double acc = 0.0;
            for (int b = 0; b < 6; ++b) {
                double ce = voigt(ec.S, c + 1, b + 1) + rf(s, hw * voigt(ec.Sp, c + 1, b + 1));
                acc += ce * ev[b];
            }
            s->sig_r[c][idx] = rf(s, acc);
        }
    RLOOP_END
    return PFGB_OK;
}

/* ------------------------------------------------------------------ */
/* phi RHS — compute_phi_rhs_kernel, cuda_kernels.cu:390-555            */
/* ------------------------------------------------------------------ */
static void phi_rhs(pfo_state *s, int coupling) {
    const pfgb_params *P = &s->p;
    const double T = P->temperature_K, sc = P->mu_reference_scale;
    const int cv = P->thermo_convex_extrapolation_enabled;
    const double shift = coupling ? P->elastic_shift_dimless : 0.0;
    double e00f[6];
    for (int c = 0; c < 6; ++c) e00f[c] = rf(s, P->eps00[c]);
    RLOOP_BEGIN(s)
        double phi = s->phi[idx];
        double hp = o_hp(phi), gp = o_gp(phi), h = o_h(phi);
        double xB = o_clamp01(s->xB[idx]);
        double f = P->W * gp;
        double muA = o_muA(xB, T, sc, cv), muB = o_muB(xB, T, sc, cv);
        double dmu = P->mu0_compound - P->v_A * muA - P->v_B * muB - shift;
        double cb = o_c_xB_phi(xB, P->Vm_alpha_0, P->dVm_alpha_dxB, P->Vm_compound, h);
        double mt = o_mu_tot_mix(muA, muB, xB, P->mu0_compound, h);
        double Vma = o_Vm_alpha(xB, P->Vm_alpha_0, P->dVm_alpha_dxB);
        double vt = P->Vm_compound - Vma + P->dVm_alpha_dxB * (xB - P->v_B);
        f += cb * hp * (dmu - cb * mt * vt);
        if (coupling) {
            double sg[6];
            for (int c = 0; c < 6; ++c) sg[c] = s->sig_r[c][idx];
            double epsc = xB * P->eps_iso_over_vB;
            double diag = -epsc + P->eps_iso_over_vB * (xB - P->v_B);
            /* the GP form of d eps0 / d phi when GP elasticity acts on phi
             * (compute_dgel_dphi_gp_point, cuda_kernels.cu:313-372, taken at
             * :513-526): the iso part weighted by 1 - h(eta), the GP strain by
             * h(eta), the whole elastic term scaled by
             * gp_elastic_derivative_scale */
            const int gp_phi = s->gp && P->gp_elastic_enabled && P->gp_elastic_active_phi;
            const double he = gp_phi ? o_h(o_clamp01(s->eta[idx])) : 0.0;
            double de[6];
            for (int c = 0; c < 3; ++c)
                de[c] = gp_phi ? hp * (P->eps00[c] + (1.0 - he) * diag - he * P->gp_eps_iso)
                               : hp * (P->eps00[c] + diag);
            for (int c = 3; c < 6; ++c) de[c] = hp * P->eps00[c];
            double dg = -(sg[0] * de[0] + sg[1] * de[1] + sg[2] * de[2]
                          + 2.0 * sg[5] * de[5] + 2.0 * sg[4] * de[4] + 2.0 * sg[3] * de[3]);
            /* eigenstrain_phi_xB_point with float eps00, stored as float */
            double e0[6];
            double omh = 1.0 - h, ec_ = xB * P->eps_iso_over_vB;
            for (int c = 0; c < 3; ++c) e0[c] = rf(s, omh * ec_ + h * e00f[c]);
            for (int c = 3; c < 6; ++c) e0[c] = rf(s, h * e00f[c]);
            double el[6], ev[6];
            for (int c = 0; c < 6; ++c) el[c] = s->eps_r[c][idx] - e0[c];
            eng(el, ev);
            double Q = 0.0;  /* compute_Q_voigt, :162-181 */
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) Q += voigt(P->S_p, a + 1, b + 1) * ev[a] * ev[b];
            f += gp_phi ? P->gp_elastic_derivative_scale * (dg + 0.5 * hp * Q) : dg + 0.5 * hp * Q;
        }
        s->rhs[idx] = f;
    RLOOP_END
}

/* phi-only minimize drive (compute_phi_rhs_minimize_kernel,
 * cuda_kernels.cu:6298-6374): double well and the elastic terms with the
 * phi-only eigenstrain h(phi) eps00 (eigenstrain_phi_only_point,
 * cuda_kernels.cu:363-384, float eps00, stored as float); no chemistry */
static void phi_rhs_phi_only(pfo_state *s) {
    const pfgb_params *P = &s->p;
    double e00f[6];
    for (int c = 0; c < 6; ++c) e00f[c] = rf(s, P->eps00[c]);
    RLOOP_BEGIN(s)
        const double phi = s->phi[idx];
        double f = P->W * o_gp(phi);
        if (P->elastic_enabled) {
            const double hp = o_hp(phi), h = o_h(phi);
            double de[6], e0[6], el[6], ev[6];
            for (int c = 0; c < 6; ++c) de[c] = hp * P->eps00[c];
            const double dg = -(s->sig_r[0][idx] * de[0] + s->sig_r[1][idx] * de[1] + s->sig_r[2][idx] * de[2] +
                                2.0 * (s->sig_r[5][idx] * de[5] + s->sig_r[4][idx] * de[4] +
                                       s->sig_r[3][idx] * de[3]));
            for (int c = 0; c < 6; ++c) e0[c] = rf(s, h * e00f[c]);
            for (int c = 0; c < 6; ++c) el[c] = s->eps_r[c][idx] - e0[c];
            eng(el, ev);
            double Q = 0.0;   /* compute_Q_voigt, :162-181 */
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) Q += voigt(P->S_p, a + 1, b + 1) * ev[a] * ev[b];
            f += dg + 0.5 * hp * Q;
        }
        s->rhs[idx] = f;
    RLOOP_END
}

/* compute_eta_rhs_kernel (non-raw-drive branch), cuda_kernels.cu:845-946 */
static void eta_rhs(pfo_state *s) {
    const pfgb_params *P = &s->p;
    const double T = P->temperature_K, sc = P->mu_reference_scale;
    const int cv = P->thermo_convex_extrapolation_enabled;
    const double xg = o_clamp_eps(P->gp_xB_fixed, 1.0e-12);
    const double g_gp = (1.0 - xg) * o_muA(xg, T, sc, cv) + xg * o_muB(xg, T, sc, cv) - P->gp_delta_g0;
    RLOOP_BEGIN(s)
        double eta = o_clamp01(s->eta[idx]);
        double phi = o_clamp01(s->phi[idx]);
        double xa = o_clamp_eps(s->xB[idx], 1.0e-12);
        double hphi = o_h(phi), hpe = o_hp(eta), gpe = o_gp(eta);
        double cref = 1.0 / o_Vm_alpha(xa, P->Vm_alpha_0, P->dVm_alpha_dxB);
        double ga = (1.0 - xa) * o_muA(xa, T, sc, cv) + xa * o_muB(xa, T, sc, cv);
        double d = cref * (1.0 - hphi) * hpe * (g_gp - ga);
        double el = 0.0;
        if (P->gp_elastic_enabled && P->gp_elastic_active_eta) {
            /* compute_dgel_deta_gp_point, cuda_kernels.cu:292-311 */
            double sh = s->sig_r[0][idx] + s->sig_r[1][idx] + s->sig_r[2][idx];
            double pre = (1.0 - o_h(phi)) * o_hp(eta);
            double ea = o_clamp01(xa) * P->eps_iso_over_vB;
            el = P->gp_elastic_derivative_scale * (-sh * (pre * (P->gp_eps_iso - ea)));
        }
        s->rhs[idx] = d + P->gp_W_eta * gpe + el;
    RLOOP_END
}

/* Test hooks (the pinning tests against the reference's own kernels): the
 * step's phi and eta right-hand sides on given fields.  sig / eps: 6 N values
 * in Voigt order xx yy zz yz xz xy. */
void pfo_test_phi_rhs(pfo_state *s, int coupling, const double *phi, const double *eta, const double *xB,
                      const double *sig, const double *eps, double *out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->phi, phi, b);
    memcpy(s->xB, xB, b);
    if (eta) memcpy(s->eta, eta, b);
    for (int c = 0; c < 6; ++c) {
        if (sig) memcpy(s->sig_r[c], sig + (size_t)c * s->N, b);
        if (eps) memcpy(s->eps_r[c], eps + (size_t)c * s->N, b);
    }
    phi_rhs(s, coupling);
    memcpy(out, s->rhs, b);
}
void pfo_test_eta_rhs(pfo_state *s, const double *eta, const double *phi, const double *xB, const double *sig,
                      double *out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->eta, eta, b);
    memcpy(s->phi, phi, b);
    memcpy(s->xB, xB, b);
    for (int c = 0; c < 6; ++c)
        if (sig) memcpy(s->sig_r[c], sig + (size_t)c * s->N, b);
    eta_rhs(s);
    memcpy(out, s->rhs, b);
}

/* ------------------------------------------------------------------ */
/* zero mode — run_pf_conserved_y_zero_mode_host, main_cuda.cu:4269-4405 */
/* ------------------------------------------------------------------ */
static int zero_mode(pfo_state *s, const double *Ystar, double Y_upper_cap, pfgb_step_stats *st) {
    const pfgb_params *P = &s->p;
    double ymin = 1e300, ymax = -1e300;
    for (size_t i = 0; i < s->N; ++i) { if (Ystar[i] < ymin) ymin = Ystar[i]; if (Ystar[i] > ymax) ymax = Ystar[i]; }
    if (!isfinite(ymin) || !isfinite(ymax)) return PFGB_ERR_ZERO_MODE;
    double lo = -P->Y_clip - ymin, hi = Y_upper_cap - ymax;
    double rnd = 128.0 * DBL_EPSILON * fmax(fmax(fabs(lo), fabs(hi)), 1.0);
    if (!isfinite(lo) || !isfinite(hi) || lo > hi + rnd) return PFGB_ERR_ZERO_MODE;
    const double target = s->target_mass;
    const double tol = P->zero_mode_tolerance_relative * fmax(fabs(target), 1.0);
#define ZM_EVAL(lam, M, D)                                                    \
    do {                                                                      \
        const double lam_ = (lam);                                            \
        RLOOP_BEGIN(s)                                                        \
            double h = o_h(s->phi[idx]);                                      \
            double a = 1.0 - h;                                               \
            double x = o_sigmoid_raw(Ystar[idx] + lam_);                      \
            s->mass_t[idx] = a * x + h * P->v_B;                              \
            s->der_t[idx] = a * x * (1.0 - x);                                \
        RLOOP_END                                                             \
        (M) = dsum(s->mass_t, s->N);                                          \
        (D) = dsum(s->der_t, s->N);                                           \
    } while (0)
    double mlo, dlo, mhi, dhi;   /* the derivatives at the bracket ends are not used */
    ZM_EVAL(lo, mlo, dlo);
    ZM_EVAL(hi, mhi, dhi);
    (void)dlo;
    (void)dhi;
    if (!isfinite(mlo) || !isfinite(mhi)) return PFGB_ERR_ZERO_MODE;
    if (mlo - target > tol || mhi - target < -tol) return PFGB_ERR_ZERO_MODE;
    double lam = fmin(fmax(0.0, lo), hi), mass, der;
    ZM_EVAL(lam, mass, der);
    double res = mass - target;
    int iters = 0, nwt = 0, bis = 0;
    for (int it = 0; it < P->zero_mode_max_iterations && fabs(res) > tol; ++it) {
        if (res < 0.0) lo = lam; else hi = lam;
        double cand = NAN;
        if (der > 0.0 && isfinite(der)) cand = lam - res / der;
        if (isfinite(cand) && cand > lo && cand < hi) ++nwt;
        else { cand = 0.5 * (lo + hi); ++bis; }
        lam = cand;
        ZM_EVAL(lam, mass, der);
        if (!isfinite(mass) || !isfinite(der)) return PFGB_ERR_ZERO_MODE;
        res = mass - target;
        iters = it + 1;
    }
#undef ZM_EVAL
    if (fabs(res) > tol) return PFGB_ERR_ZERO_MODE;
    for (size_t i = 0; i < s->N; ++i) {
        double y = Ystar[i] + lam;
        if (!isfinite(y) || y < -P->Y_clip || y > Y_upper_cap) return PFGB_ERR_ZERO_MODE;
    }
    RLOOP_BEGIN(s)
        double y = Ystar[idx] + lam;
        s->Y[idx] = y;
        s->xB[idx] = o_sigmoid_raw(y);
    RLOOP_END
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

/* two_phase_storage_exact_Y_update_kernel, cuda_kernels.cu:2859-2921: the
 * point update of the composition from divJ, Y^n, phi^n and phi^{n+1} */
static void storage_exact_update(pfo_state *s, double dt) {
    const pfgb_params *P = &s->p;
    RLOOP_BEGIN(s)
        const double ho = o_h(o_clamp01(s->phi_n[idx])), hn = o_h(o_clamp01(s->phi[idx]));
        const double xo = o_sigmoid(s->Y_n[idx], P->Y_clip, P->xB_eps);
        const double Ct = (1.0 - ho) * xo + ho * P->v_B + dt * s->divJ[idx];
        const double han = 1.0 - hn;
        const int small = !(han >= P->gp_h_alpha_eps);
        double xt = xo;
        if (!small && isfinite(Ct)) xt = (Ct - hn * P->v_B) / han;
        const int bad = small || !isfinite(xt) || xt < P->xB_eps || xt > 1.0 - P->xB_eps;
        const double y = o_logit(bad ? xo : xt, P->xB_eps, P->Y_clip);
        s->Y[idx] = y;
        s->xB[idx] = o_sigmoid(y, P->Y_clip, P->xB_eps);
        s->dYdt[idx] = (y - s->Y_n[idx]) / dt;
    RLOOP_END
}

/* test hook (the pinning tests): the storage-exact update on given fields */
void pfo_test_storage_exact(pfo_state *s, double dt, const double *divJ, const double *phi_new,
                            const double *phi_old, const double *Y_old, double *Y, double *xB) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->divJ, divJ, b);
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->Y_n, Y_old, b);
    storage_exact_update(s, dt);
    memcpy(Y, s->Y, b);
    memcpy(xB, s->xB, b);
}

/* one flux component J_a = M g_a over s->scr in place, g_a the unnormalised
 * inverse transform of i k_a mu (compute_flux_single_component_kernel,
 * cuda_kernels.cu:1985-2037; gp_zone: compute_flux_single_component_gp_kernel,
 * :2039-2110), the mobility from the composition of Y^n in s->xB_prev */
static void flux_field(pfo_state *s, const double *phiY, const double *etaY) {
    const pfgb_params *P = &s->p;
    const double T = P->temperature_K, sc = P->mu_reference_scale;
    const int cv = P->thermo_convex_extrapolation_enabled;
    RLOOP_BEGIN(s)
        double g = s->scr[idx] * s->invN;
        double M;
        if (s->gp) {   /* compute_flux_single_component_gp_kernel, :2039 */
            double hb = o_h(phiY[idx]), he = o_h(etaY[idx]);
            double hg = (1.0 - hb) * he, ha = (1.0 - hb) * (1.0 - he);
            double Ga = o_gamma(s->xB_prev[idx], 0.0, P->Vm_alpha_0, P->dVm_alpha_dxB,
                                P->Vm_compound, T, sc, cv);
            double Ma = o_meff(P->D_alpha, Ga);
            M = ha * Ma + hg * P->gp_M_GP + hb * P->gp_M_beta;
        } else if (P->pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT) {
            /* compute_flux_single_component_q_kernel, :2014-2037: the matrix
             * channel alone, (1 - h) M_alpha with G_alpha at h = 0 */
            double a = 1.0 - o_h(o_clamp01(phiY[idx]));
            double Ga = o_gamma(s->xB_prev[idx], 0.0, P->Vm_alpha_0, P->dVm_alpha_dxB,
                                P->Vm_compound, T, sc, cv);
            M = a * o_meff(P->D_alpha, Ga);
        } else {       /* compute_flux_single_component_kernel, :1985 */
            double h = o_h(phiY[idx]);
            double Dm = o_Dmix(h, P->D_alpha, P->D_compound);
            double G = o_gamma(s->xB_prev[idx], h, P->Vm_alpha_0, P->dVm_alpha_dxB,
                               P->Vm_compound, T, sc, cv);
            M = o_meff(Dm, G);
        }
        s->scr[idx] = M * g;
    RLOOP_END
}

/* test hook (the pinning tests): one flux component on given fields; g is
 * the normalised gradient */
void pfo_test_flux(pfo_state *s, const double *g, const double *phiY, const double *etaY, const double *xB_prev,
                   double *J) {
    const size_t b = sizeof(double) * s->N;
    for (size_t i = 0; i < s->N; ++i) s->scr[i] = g[i] * (double)s->N;
    memcpy(s->xB_prev, xB_prev, b);
    flux_field(s, phiY, etaY);
    memcpy(J, s->scr, b);
}

/* the x split's right-hand side S - m Lap(x^n) with the storage source
 * S = divJ / (1 - h^{n+1}) where the matrix storage reaches its floor
 * (compute_xB_storage_rhs_kernel, cuda_kernels.cu:2922-2951); lapY holds the
 * unnormalised inverse transform of -k^2 x^n */
static void xsplit_source(pfo_state *s, double mDx) {
    const pfgb_params *P = &s->p;
    RLOOP_BEGIN(s)
        const double lap = s->lapY[idx] * s->invN;
        const double ha = 1.0 - o_h(o_clamp01(s->phi[idx]));
        const double rate = ha >= P->pf_matrix_storage_floor ? s->divJ[idx] / ha : 0.0;
        s->rhs[idx] = rate - mDx * lap;
    RLOOP_END
}

/* the x split's new composition from the unnormalised inverse transform in
 * scr (xB_normalize_clamp_and_logit_kernel, :2953-2973) */
static void xsplit_final(pfo_state *s, double dt) {
    const pfgb_params *P = &s->p;
    RLOOP_BEGIN(s)
        double x = s->scr[idx] * s->invN;
        if (!isfinite(x)) x = s->xB[idx];
        x = fmin(fmax(x, P->xB_eps), 1.0 - P->xB_eps);
        double y = o_logit(x, P->xB_eps, P->Y_clip);
        y = fmin(fmax(y, -P->Y_clip), P->Y_clip);
        s->Y[idx] = y;
        s->xB[idx] = o_sigmoid(y, P->Y_clip, P->xB_eps);
        s->dYdt[idx] = (y - s->Y_n[idx]) / dt;
    RLOOP_END
}

/* test hooks (the pinning tests) for the two x-split functions; lap and x
 * are normalised */
void pfo_test_xsplit_source(pfo_state *s, double mDx, const double *divJ, const double *phi_new,
                            const double *lap, double *rhs) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->divJ, divJ, b);
    memcpy(s->phi, phi_new, b);
    for (size_t i = 0; i < s->N; ++i) s->lapY[i] = lap[i] * (double)s->N;
    xsplit_source(s, mDx);
    memcpy(rhs, s->rhs, b);
}
void pfo_test_xsplit_final(pfo_state *s, double dt, const double *x, const double *xB_old, double *Y, double *xB) {
    const size_t b = sizeof(double) * s->N;
    for (size_t i = 0; i < s->N; ++i) s->scr[i] = x[i] * (double)s->N;
    memcpy(s->xB, xB_old, b);
    memset(s->Y_n, 0, b);
    xsplit_final(s, dt);
    memcpy(Y, s->Y, b);
    memcpy(xB, s->xB, b);
}

/* q_transport_projection_split (main_cuda.cu:27781-27783): the matrix
 * storage q = (1 - h) x of the conserved composition is the evolved
 * coordinate.  Bounds and tolerances as the reference's calls: feasibility
 * and bound tolerance 1e-12, redistribution radius 8. */
#define Q_TOL 1.0e-12

/* initialize_q_alpha_kernel / sync_q_from_phi_xB_kernel, cuda_kernels.cu:2975-2984, 3107-3116 */
static void q_from_phi_xB(pfo_state *s) {
    RLOOP_BEGIN(s)
        s->q[idx] = (1.0 - o_h(o_clamp01(s->phi[idx]))) * s->xB[idx];
    RLOOP_END
}

/* the bounded context x = q / (1 - h) -> Y -> x (the tail shared by
 * q_normalize_validate_and_reconstruct_kernel :3032-3069 and
 * q_explicit_transport_and_reconstruct_kernel :3071-3105) */
static void q_context(pfo_state *s, size_t idx, double q, double alpha) {
    const pfgb_params *P = &s->p;
    double x = s->xB[idx];
    if (alpha > 1.0e-14) x = q / alpha;
    x = fmin(fmax(x, P->xB_eps), 1.0 - P->xB_eps);
    double y = o_logit(x, P->xB_eps, P->Y_clip);
    y = fmin(fmax(y, -P->Y_clip), P->Y_clip);
    s->xB[idx] = o_sigmoid(y, P->Y_clip, P->xB_eps);
    s->Y[idx] = y;
}

/* q_normalize_validate_and_reconstruct_kernel with invN = 1, :3032-3069 */
static void q_reconstruct(pfo_state *s) {
    RLOOP_BEGIN(s)
        const double alpha = 1.0 - o_h(o_clamp01(s->phi[idx]));
        double q = s->q[idx];
        q = isfinite(q) ? fmin(fmax(q, 0.0), alpha) : 0.0;
        s->q[idx] = q;
        q_context(s, idx, q, alpha);
    RLOOP_END
}

/* the phase substep's storage transfer q -= (h_new - h_old) v_B
 * (apply_local_phase_storage_transfer_q_kernel, :2989-3019); where it is
 * infeasible anywhere the whole phi substep is rejected: phi returns to
 * phi^n and q is rebuilt from it (main_cuda.cu:30241-30266).  Then the
 * context is refreshed (:30271-30274). */
static long long q_phase_cells(pfo_state *s) {
    const pfgb_params *P = &s->p;
    long long bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
    for (long long i = 0; i < (long long)s->N; ++i) {
        const double ho = o_h(o_clamp01(s->phi_n[i])), hn = o_h(o_clamp01(s->phi[i]));
        const double an = 1.0 - hn;
        const double qn = s->q[i] - (hn - ho) * P->v_B;
        if (!isfinite(qn) || qn < -Q_TOL || qn > an + Q_TOL) { ++bad; continue; }
        s->q[i] = fmin(fmax(qn, 0.0), an);
    }
    return bad;
}
static void q_phase(pfo_state *s) {
    const long long bad = q_phase_cells(s);
    s->q_rejected = bad > 0;
    if (bad) {
        memcpy(s->phi, s->phi_n, sizeof(double) * s->N);
        q_from_phi_xB(s);
    }
    q_reconstruct(s);
}

/* the host's local redistribution of out-of-bounds transport
 * (q_transport_conservative_local_redistribution, main_cuda.cu:22362-22456):
 * each cell's trial q + dt divJ is bounded to [0, 1 - h]; in cell order the
 * excess (or deficit) goes to the cells of growing Chebyshev shells around
 * it, up to radius 8, within their capacity (1 - h - q) or storage (q).
 * Returns 0 when an amount stays unresolved beyond the tolerance. */
static int q_redistribute(pfo_state *s, double dt, int *violating) {
    const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz, R = 8;
    double *alpha = s->mass_t, *res = s->der_t;
    int nv = 0;
    for (size_t i = 0; i < s->N; ++i) {
        alpha[i] = 1.0 - o_h(o_clamp01(s->phi[i]));
        const double trial = s->q_before[i] + dt * s->divJ[i];
        const double b = fmin(fmax(trial, 0.0), alpha[i]);
        s->q[i] = b;
        res[i] = trial - b;
        if (!isfinite(trial) || fabs(res[i]) > Q_TOL) ++nv;
    }
    double unresolved = 0.0;
    for (size_t i = 0; i < s->N; ++i) {
        double amt = res[i];
        if (!isfinite(amt)) { unresolved = INFINITY; continue; }
        if (fabs(amt) <= Q_TOL) continue;
        const int k0 = (int)(i % Nz), j0 = (int)((i / Nz) % Ny), i0 = (int)(i / ((size_t)Nz * Ny));
        for (int r = 1; r <= R && fabs(amt) > Q_TOL; ++r)
            for (int di = -r; di <= r && fabs(amt) > Q_TOL; ++di)
                for (int dj = -r; dj <= r && fabs(amt) > Q_TOL; ++dj)
                    for (int dk = -r; dk <= r && fabs(amt) > Q_TOL; ++dk) {
                        const int m = abs(di) > abs(dj) ? abs(di) : abs(dj);
                        if ((m > abs(dk) ? m : abs(dk)) != r) continue;
                        const size_t n = ((size_t)((i0 + di + Nx) % Nx) * Ny + (size_t)((j0 + dj + Ny) % Ny)) * Nz +
                                         (size_t)((k0 + dk + Nz) % Nz);
                        if (amt > 0.0) {
                            const double cap = alpha[n] - s->q[n];
                            if (cap <= 0.0) continue;
                            const double mv = fmin(amt, cap);
                            s->q[n] += mv;
                            amt -= mv;
                        } else {
                            const double av = s->q[n];
                            if (av <= 0.0) continue;
                            const double mv = fmin(-amt, av);
                            s->q[n] -= mv;
                            amt += mv;
                        }
                    }
        unresolved += fabs(amt);
    }
    *violating = nv;
    return isfinite(unresolved) && unresolved <= Q_TOL * fmax(1.0, (double)nv);
}

/* the composition update of the q split from divJ (real, normalised):
 * q_explicit_transport_and_reconstruct_kernel (:3071-3105), the local
 * redistribution and q_normalize_validate_and_reconstruct_kernel when a cell
 * left its bounds (main_cuda.cu:30648-30707), sync_q_from_phi_xB_kernel
 * (:31227-31229) and update_dY_dt_prev_kernel */
static long long q_transport_cells(pfo_state *s, double dt) {
    long long viol = 0;
#pragma omp parallel for schedule(static) reduction(+ : viol)
    for (long long i = 0; i < (long long)s->N; ++i) {
        const double alpha = 1.0 - o_h(o_clamp01(s->phi[i]));
        const double qt = s->q[i] + dt * s->divJ[i];
        if (!isfinite(qt) || qt < -Q_TOL || qt > alpha + Q_TOL) ++viol;
        const double q = isfinite(qt) ? fmin(fmax(qt, 0.0), alpha) : 0.0;
        s->q[i] = q;
        q_context(s, (size_t)i, q, alpha);
    }
    return viol;
}
static int q_transport(pfo_state *s, double dt) {
    memcpy(s->q_before, s->q, sizeof(double) * s->N);
    const long long viol = q_transport_cells(s, dt);
    s->q_redistributed = 0;
    if (viol) {
        int nv = 0;
        if (!q_redistribute(s, dt, &nv)) return PFGB_ERR_NONCONVERGED;
        s->q_redistributed = nv;
        q_reconstruct(s);
    }
    q_from_phi_xB(s);
    RLOOP_BEGIN(s) s->dYdt[idx] = (s->Y[idx] - s->Y_n[idx]) / dt; RLOOP_END
    return PFGB_OK;
}

static void mu_field(pfo_state *s, const double *phiY, const double *etaY);

/* PF-only conservative composition modes (pf_composition_mode,
 * main_cuda.cu:27784-27792): the storage C = q + h v_B (ctot) or q (qalpha)
 * moved by limited pairwise face transfers; kernels cuda_kernels.cu:3117-3288 */

/* h^-1 by 60 bisections on [0, 1] (h_inverse_bisection_device, :85-97) */
static double h_inverse_bisect(double target) {
    if (target <= 0.0) return 0.0;
    if (target >= 1.0) return 1.0;
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 60; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (o_h(mid) < target) lo = mid; else hi = mid;
    }
    return 0.5 * (lo + hi);
}

/* initialize_conservative_storage_kernel, :3123-3132 */
static void cons_init(pfo_state *s) {
    const pfgb_params *P = &s->p;
    const int ctot = P->pf_composition_mode == PFGB_COMPOSITION_CTOT;
    RLOOP_BEGIN(s)
        const double h = o_h(o_clamp01(s->phi[idx]));
        const double q = (1.0 - h) * o_clamp01(s->xB[idx]);
        s->cstore[idx] = ctot ? q + h * P->v_B : q;
    RLOOP_END
}

/* the matrix composition of a cell from its storage: x = q / (1 - h), the
 * equilibrium composition where the matrix vanishes or x is not finite,
 * bounded to [eps, 1 - eps], and its logit (the tail shared by
 * reconstruct_conservative_context_kernel :3134-3159 and
 * constrain_phase_and_reconstruct_conservative_kernel :3239-3288) */
static void cons_x(pfo_state *s, size_t idx, double q, double alpha) {
    const pfgb_params *P = &s->p;
    double x = P->xB_eq_matrix;
    if (alpha > P->pf_conservative_beta_support_eps) x = q / alpha;
    if (!isfinite(x)) x = P->xB_eq_matrix;
    x = fmin(fmax(x, P->xB_eps), 1.0 - P->xB_eps);
    s->xB[idx] = x;
    s->Y[idx] = o_logit(x, P->xB_eps, P->Y_clip);
}

/* reconstruct_conservative_context_kernel, :3134-3159 */
static void cons_context(pfo_state *s, const double *phi) {
    const pfgb_params *P = &s->p;
    const int ctot = P->pf_composition_mode == PFGB_COMPOSITION_CTOT;
    RLOOP_BEGIN(s)
        const double h = o_h(o_clamp01(phi[idx]));
        const double alpha = fmax(1.0 - h, 0.0);
        const double q = ctot ? s->cstore[idx] - h * P->v_B : s->cstore[idx];
        cons_x(s, idx, q, alpha);
    RLOOP_END
}

/* one checkerboard sweep of the pairwise face transfer along an axis: the
 * face between each cell of the given coordinate parity and its + neighbour
 * (periodic), matrix-channel mobilities (1 - h) M_alpha joined harmonically,
 * transfer dt M (mu_i - mu_j) / dx^2 (damped by the backward-Euler factor
 * 1 + dt M / dx^2 max(G_i / a_i + G_j / a_j, 0)), limited by both cells'
 * storage bounds [h v_B, h v_B + (1 - h)] (ctot) or [0, 1 - h] (qalpha)
 * (pairwise_conservative_face_sweep_kernel, :3161-3237).  Every cell is on one
 * face of a sweep, so the faces are independent. */
static long long cons_sweep(pfo_state *s, int axis, int parity, double spacing) {
    const pfgb_params *P = &s->p;
    const int ctot = P->pf_composition_mode == PFGB_COMPOSITION_CTOT;
    const int be = P->pf_conservative_flux_strategy == PFGB_CONS_FLUX_BACKWARD_EULER;
    const double T = P->temperature_K, sc = P->mu_reference_scale, dt = P->dt;
    const int cv = P->thermo_convex_extrapolation_enabled;
    const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz;
    long long limited = 0;
#pragma omp parallel for schedule(static) reduction(+ : limited)
    for (long long idx = 0; idx < (long long)s->N; ++idx) {
        const int k = (int)(idx % Nz), t = (int)(idx / Nz), j = t % Ny, i = t / Ny;
        const int coord = axis == 0 ? i : (axis == 1 ? j : k);
        if ((coord & 1) != parity) continue;
        int ni = i, nj = j, nk = k;
        if (axis == 0) ni = i + 1 == Nx ? 0 : i + 1;
        else if (axis == 1) nj = j + 1 == Ny ? 0 : j + 1;
        else nk = k + 1 == Nz ? 0 : k + 1;
        const size_t n = ((size_t)ni * Ny + nj) * Nz + nk;
        const double hi = o_h(o_clamp01(s->phi_n[idx])), hj = o_h(o_clamp01(s->phi_n[n]));
        const double ai = fmax(1.0 - hi, 0.0), aj = fmax(1.0 - hj, 0.0);
        const double xi = fmin(fmax(s->xB[idx], 1e-12), 1.0 - 1e-12), xj = fmin(fmax(s->xB[n], 1e-12), 1.0 - 1e-12);
        const double Gi = o_gamma(xi, 0.0, P->Vm_alpha_0, P->dVm_alpha_dxB, P->Vm_compound, T, sc, cv);
        const double Gj = o_gamma(xj, 0.0, P->Vm_alpha_0, P->dVm_alpha_dxB, P->Vm_compound, T, sc, cv);
        const double Mi = ai * o_meff(P->D_alpha, Gi), Mj = aj * o_meff(P->D_alpha, Gj);
        const double Mf = (Mi > 0.0 && Mj > 0.0) ? 2.0 * Mi * Mj / (Mi + Mj) : 0.0;
        const double inv2 = 1.0 / (spacing * spacing);
        double tr = dt * Mf * (s->mu[idx] - s->mu[n]) * inv2;
        if (be && Mf > 0.0) {
            const double di = Gi / fmax(ai, 1.0e-14), dj = Gj / fmax(aj, 1.0e-14);
            tr /= 1.0 + dt * Mf * inv2 * fmax(di + dj, 0.0);
        }
        const double si = s->cstore[idx], sj = s->cstore[n];
        const double loi = ctot ? hi * P->v_B : 0.0, loj = ctot ? hj * P->v_B : 0.0;
        const double upi = ctot ? hi * P->v_B + ai : ai, upj = ctot ? hj * P->v_B + aj : aj;
        const double raw = tr;
        if (tr >= 0.0) {
            tr = fmin(tr, fmax(si - loi, 0.0));
            tr = fmin(tr, fmax(upj - sj, 0.0));
        } else {
            const double mag = fmin(-tr, fmax(sj - loj, 0.0));
            tr = -fmin(mag, fmax(upi - si, 0.0));
        }
        if (fabs(tr - raw) > P->pf_conservative_bound_tol) ++limited;
        s->cstore[idx] = si - tr;
        s->cstore[n] = sj + tr;
    }
    return limited;
}

/* the storage constraint on the new phi and the context from it
 * (constrain_phase_and_reconstruct_conservative_kernel, :3239-3288): h is
 * capped at C / v_B (phi by bisection); a cell whose storage would leave its
 * bounds keeps phi^n and is counted (the host rejects the step); qalpha
 * stores q for the new h.  Returns the rejected cells; *constrained: the
 * capped ones. */
static long long cons_constrain(pfo_state *s, long long *constrained) {
    const pfgb_params *P = &s->p;
    const int ctot = P->pf_composition_mode == PFGB_COMPOSITION_CTOT;
    const double tol = P->pf_conservative_bound_tol, vB = P->v_B;
    long long bad = 0, capped = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad, capped)
    for (long long i = 0; i < (long long)s->N; ++i) {
        const double po = o_clamp01(s->phi_n[i]);
        const double ho = o_h(po);
        const double C = ctot ? s->cstore[i] : s->cstore[i] + ho * vB;
        double phi = o_clamp01(s->phi[i]);
        double h = o_h(phi);
        const double hmax = vB > 0.0 ? fmin(fmax(C / vB, 0.0), 1.0) : 1.0;
        if (h > hmax + tol) {
            phi = h_inverse_bisect(hmax);
            h = o_h(phi);
            ++capped;
        }
        double alpha = fmax(1.0 - h, 0.0);
        double q = C - h * vB;
        if (!isfinite(q) || q < -tol || q > alpha + tol) {
            ++bad;
            phi = po;
            h = ho;
            alpha = fmax(1.0 - h, 0.0);
            q = C - h * vB;
        }
        s->phi[i] = phi;
        if (!ctot) s->cstore[i] = q;
        double x = P->xB_eq_matrix;
        if (alpha > P->pf_conservative_beta_support_eps) x = q / alpha;
        if (!isfinite(x)) { x = P->xB_eq_matrix; ++bad; }
        x = fmin(fmax(x, P->xB_eps), 1.0 - P->xB_eps);
        s->xB[i] = x;
        s->Y[i] = o_logit(x, P->xB_eps, P->Y_clip);
    }
    *constrained = capped;
    return bad;
}

/* the transport half of a conservative step, before the elastic solve
 * (main_cuda.cu:28486-28545): context at phi^n, mu there, the six sweeps
 * (x, y, z; parity 0 then 1), the context again */
static void cons_transport(pfo_state *s) {
    const pfgb_params *P = &s->p;
    cons_context(s, s->phi_n);
    mu_field(s, s->phi_n, s->eta);
    const double sp[3] = {P->dx, P->dy, P->dz};
    long long lim = 0;
    for (int a = 0; a < 3; ++a)
        for (int par = 0; par < 2; ++par) lim += cons_sweep(s, a, par, sp[a]);
    s->cons_limited = lim;
    cons_context(s, s->phi_n);
}

/* test hooks (the pinning tests) for the conservative modes' functions */
void pfo_test_cons_init(pfo_state *s, const double *phi, const double *xB, double *storage) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->phi, phi, b);
    memcpy(s->xB, xB, b);
    cons_init(s);
    memcpy(storage, s->cstore, b);
}
void pfo_test_cons_context(pfo_state *s, const double *storage, const double *phi, double *xB, double *Y) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->cstore, storage, b);
    cons_context(s, phi);
    memcpy(xB, s->xB, b);
    memcpy(Y, s->Y, b);
}
long long pfo_test_cons_sweep(pfo_state *s, double *storage, const double *mu, const double *phi, const double *xB,
                              int axis, int parity, double spacing) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->cstore, storage, b);
    memcpy(s->mu, mu, b);
    memcpy(s->phi_n, phi, b);
    memcpy(s->xB, xB, b);
    const long long lim = cons_sweep(s, axis, parity, spacing);
    memcpy(storage, s->cstore, b);
    return lim;
}
long long pfo_test_cons_constrain(pfo_state *s, double *phi_new, const double *phi_old, double *storage, double *xB,
                                  double *Y, long long *capped) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->cstore, storage, b);
    const long long bad = cons_constrain(s, capped);
    memcpy(phi_new, s->phi, b);
    memcpy(storage, s->cstore, b);
    memcpy(xB, s->xB, b);
    memcpy(Y, s->Y, b);
    return bad;
}

/* test hooks (the pinning tests) for the q split's per-cell functions */
long long pfo_test_q_phase(pfo_state *s, const double *phi_new, const double *phi_old, const double *q_in,
                           double *q_out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->q, q_in, b);
    const long long bad = q_phase_cells(s);
    memcpy(q_out, s->q, b);
    return bad;
}
long long pfo_test_q_transport(pfo_state *s, double dt, const double *q_in, const double *divJ, const double *phi,
                               const double *xB_in, double *q_out, double *xB_out, double *Y_out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->q, q_in, b);
    memcpy(s->divJ, divJ, b);
    memcpy(s->phi, phi, b);
    memcpy(s->xB, xB_in, b);
    const long long viol = q_transport_cells(s, dt);
    memcpy(q_out, s->q, b);
    memcpy(xB_out, s->xB, b);
    memcpy(Y_out, s->Y, b);
    return viol;
}
void pfo_test_q_reconstruct(pfo_state *s, const double *q_in, const double *phi, const double *xB_in, double *q_out,
                            double *xB_out, double *Y_out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->q, q_in, b);
    memcpy(s->phi, phi, b);
    memcpy(s->xB, xB_in, b);
    q_reconstruct(s);
    memcpy(q_out, s->q, b);
    memcpy(xB_out, s->xB, b);
    memcpy(Y_out, s->Y, b);
}

/* test hook (the pinning tests): the 2/3 dealias rule on a given half
 * spectrum (Nk complex values, in place) */
void pfo_test_dealias(pfo_state *s, double *k) {
    memcpy(s->scr_k, k, sizeof(cpx) * s->Nk);
    dealias(s, s->scr_k);
    memcpy(k, s->scr_k, sizeof(cpx) * s->Nk);
}

/* mu of the flux, in place of Y^n's composition (compute_mu_x_kernel,
 * cuda_kernels.cu:1266-1324; gp_zone: compute_mu_C_gp_kernel, :1326-1366);
 * also xB = sigmoid(Y) */
static void mu_field(pfo_state *s, const double *phiY, const double *etaY) {
    pfgb_params *P = &s->p;
    const double T = P->temperature_K, sc = P->mu_reference_scale;
    const int cv = P->thermo_convex_extrapolation_enabled;
    (void)etaY;
    RLOOP_BEGIN(s)
        double Yv = s->Y[idx];
        double xB = o_sigmoid(Yv, P->Y_clip, P->xB_eps);
        s->xB[idx] = xB;
        double muA = o_muA(xB, T, sc, cv), muB = o_muB(xB, T, sc, cv);
        double mu;
        if (s->gp) {   /* compute_mu_C_gp_kernel, :1326-1366 */
            double cref = 1.0 / o_Vm_alpha(xB, P->Vm_alpha_0, P->dVm_alpha_dxB);
            mu = cref * (muB - muA);
        } else {       /* compute_mu_x_kernel, :1266-1324 */
            double h = o_h(phiY[idx]);
            double cb = o_c_xB_phi(xB, P->Vm_alpha_0, P->dVm_alpha_dxB, P->Vm_compound, h);
            double mt = o_mu_tot_mix(muA, muB, xB, P->mu0_compound, h);
            mu = cb * (muB - muA - cb * mt * P->dVm_alpha_dxB);
        }
        if (P->elastic_enabled) {
            double sh = s->sig_r[0][idx] + s->sig_r[1][idx] + s->sig_r[2][idx];
            mu += -P->eps_iso_over_vB * sh;
        }
        s->mu[idx] = mu;
    RLOOP_END
}

/* ------------------------------------------------------------------ */
/* GP storage coupling (gp_zone with gp_barrier_only_mode = 0 or       */
/* enable_legacy_gp_storage_coupling = 1, gp_storage_coupling_enabled, */
/* main_cuda.cu:16767-16772): the conserved composition is             */
/* xBtot_gp = h_alpha x + h_GP x_GP + h_beta                           */
/* ------------------------------------------------------------------ */
static int gp_coupled(const pfo_state *s) {
    return s->gp && (s->p.enable_legacy_gp_storage_coupling || !s->p.gp_barrier_only_mode);
}

/* phase_fractions_gp, phase_functions.h:27-42 (phi and eta as given) */
static void o_gpfrac(double phi, double eta, double *ha, double *hg, double *hb) {
    const double hp = o_h(phi), he = o_h(eta);
    *hb = hp;
    *hg = (1.0 - hp) * he;
    *ha = (1.0 - hp) * (1.0 - he);
}

/* the matrix composition recovered from a storage target, and whether it
 * lies in [x_min, x_max] (gp_recovered_xB_valid_device, cuda_kernels.cu:1100-1120) */
static int gp_recovered_valid(double tot, double hb, double A, double hg, double xg, double xmin, double xmax,
                              double eps_h, double *xr) {
    if (!isfinite(tot) || !isfinite(hb) || !isfinite(A) || !isfinite(hg)) return 0;
    if (A < 0.0) return 0;
    if (hg < 0.0 || hg > A) return 0;
    const double ha = A - hg;
    if (!(ha >= eps_h)) return 0;
    const double num = tot - hg * xg - hb;
    if (!isfinite(num)) return 0;
    const double x = num / ha;
    if (!isfinite(x)) return 0;
    if (xr) *xr = x;
    return x >= xmin && x <= xmax;
}

/* the largest GP fraction in [0, min(h_GP, A)] whose recovered composition
 * is valid, by 80 bisections (gp_limited_hGP_device, :1122-1149) */
static double gp_limited_hgp(double tot, double hb, double A, double hg_tent, double xg, double xmin, double xmax,
                             double eps_h) {
    if (!isfinite(tot) || !isfinite(hb) || !isfinite(A) || !isfinite(hg_tent)) return 0.0;
    const double hi0 = fmin(fmax(hg_tent, 0.0), fmax(A, 0.0));
    double xr = 0.0;
    if (gp_recovered_valid(tot, hb, A, hi0, xg, xmin, xmax, eps_h, &xr)) return hi0;
    double lo = 0.0, hi = hi0;
    for (int it = 0; it < 80; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (gp_recovered_valid(tot, hb, A, mid, xg, xmin, xmax, eps_h, &xr)) lo = mid; else hi = mid;
    }
    return lo;
}

/* the eta feasibility check after the flux (gp_eta_feasibility_and_limiter_kernel,
 * :1151-1250): eta clamped to [0, 1]; with the local_clip limiter, where the
 * storage target xBtot_gp^n + dt divJ cannot be met by a matrix composition
 * in [xB_eps, 1 - xB_eps] under the tentative GP fraction, the GP fraction is
 * lowered to the largest feasible one and eta follows by inverting h.  x^n is
 * the composition of Y^n (s->xB_gp_old).  Returns the limited cells. */
static long long gp_eta_feasibility(pfo_state *s, double dt, int limiter) {
    const pfgb_params *P = &s->p;
    const double xmin = P->xB_eps, xmax = 1.0 - P->xB_eps, eps_h = P->gp_h_alpha_eps, xg = P->gp_xB_fixed;
    long long limited = 0;
#pragma omp parallel for schedule(static) reduction(+ : limited)
    for (long long i = 0; i < (long long)s->N; ++i) {
        const double et = o_clamp01(s->eta[i]);
        const double pnew = o_clamp01(s->phi[i]), pold = o_clamp01(s->phi_n[i]);
        const double xo = o_clamp_eps(s->xB_gp_old[i], xmin);
        double hao, hgo, hbo;
        o_gpfrac(pold, o_clamp01(s->eta_prev[i]), &hao, &hgo, &hbo);
        const double hpn = o_h(pnew);
        const double A = fmax(1.0 - hpn, 0.0);
        const double hg_tent = A * o_h(et);
        const double tot_old = xo + hgo * (xg - xo) + hbo * (1.0 - xo);
        const double target = tot_old + dt * s->divJ[i];
        double xr = 0.0;
        const int valid = gp_recovered_valid(target, hpn, A, hg_tent, xg, xmin, xmax, eps_h, &xr);
        double ef = et;
        if (limiter && A > eps_h && hg_tent > 0.0 && !valid) {
            const double hgf = gp_limited_hgp(target, hpn, A, hg_tent, xg, xmin, xmax, eps_h);
            double allowed = o_clamp01(hgf / fmax(A, eps_h));
            ef = h_inverse_bisect(allowed);
            if (!isfinite(ef)) ef = 0.0;
            ef = o_clamp01(ef);
            if (fabs(et - ef) > 0.0) ++limited;
        }
        s->eta[i] = ef;
    }
    return limited;
}

/* the storage-consistent point updates of Y (gp_y_update_mode storage_exact,
 * gp_storage_exact_Y_update_kernel :2746-2857, and picard_storage,
 * gp_picard_storage_Y_update_kernel :3290-3370, repeated gp_y_picard_iters
 * times from the guess Y^n); the fractions at (phi^n, eta^n) and
 * (phi^{n+1}, eta^{n+1}); Y capped at +-Y_clip */
static void gp_storage_update(pfo_state *s, double dt) {
    const pfgb_params *P = &s->p;
    const double eps = P->xB_eps, Yc = P->Y_clip, xg = P->gp_xB_fixed;
    const int picard = P->gp_y_update_mode == PFGB_GP_Y_PICARD_STORAGE;
    const int iters = P->gp_y_picard_iters > 0 ? P->gp_y_picard_iters : 1;
    RLOOP_BEGIN(s)
        double hao, hgo, hbo, han, hgn, hbn;
        o_gpfrac(s->phi_n[idx], s->eta_prev[idx], &hao, &hgo, &hbo);
        o_gpfrac(s->phi[idx], s->eta[idx], &han, &hgn, &hbn);
        const double xo = o_sigmoid(s->Y_n[idx], Yc, eps);
        const double So = hgo * (xg - xo) + hbo * (1.0 - xo);
        if (!picard) {
            const double target = xo + So + dt * s->divJ[idx];
            if (!isfinite(target)) {
                s->Y[idx] = s->Y_n[idx];
                s->xB[idx] = xo;
            } else {
                double xu = xo;
                if (!(han < P->gp_h_alpha_eps)) xu = (target - hgn * xg - hbn) / han;
                if (!isfinite(xu)) xu = xo;
                double xf = xu;
                if (xf < eps) xf = eps;
                if (xf > 1.0 - eps) xf = 1.0 - eps;
                double y = o_logit(xf, eps, Yc);
                if (y > Yc) y = Yc;
                if (y < -Yc) y = -Yc;
                s->Y[idx] = y;
                s->xB[idx] = o_sigmoid(y, Yc, eps);
            }
        } else {
            const int small = han < fmax(eps, 1.0e-8);
            double yg = s->Y[idx];
            for (int it = 0; it < iters; ++it) {
                const double xgs = o_sigmoid(yg, Yc, eps);
                double xu = xo;
                if (!small) {
                    const double Sg = hgn * (xg - xgs) + hbn * (1.0 - xgs);
                    xu = xo + dt * (s->divJ[idx] - (Sg - So) / dt);
                }
                double xf = xu;
                if (xf < eps) xf = eps;
                if (xf > 1.0 - eps) xf = 1.0 - eps;
                double y = o_logit(xf, eps, Yc);
                if (y > Yc) y = Yc;
                if (y < -Yc) y = -Yc;
                yg = y;
            }
            s->Y[idx] = yg;
            s->xB[idx] = o_sigmoid(yg, Yc, eps);
        }
    RLOOP_END
}

/* sum of h_alpha D_alpha x (1 - x) over the cells (reduce_sum_DY_gp_kernel,
 * :3923-3955), the fractions at the given phi and eta */
static double gp_sum_DY(pfo_state *s, const double *phiY, const double *etaY) {
    const pfgb_params *P = &s->p;
    RLOOP_BEGIN(s)
        double ha, hg, hb;
        o_gpfrac(phiY[idx], etaY[idx], &ha, &hg, &hb);
        const double x = o_sigmoid(s->Y[idx], 20.0, 1e-12);
        s->mass_t[idx] = ha * P->D_alpha * (x * (1.0 - x));
    RLOOP_END
    return dsum(s->mass_t, s->N);
}

/* test hooks (the pinning tests) for the GP storage coupling's functions;
 * inputs are copied into the state, outputs read back */
void pfo_test_gp_storage(pfo_state *s, double dt, const double *divJ, const double *phi_new, const double *phi_old,
                         const double *eta_new, const double *eta_old, const double *Y_old, const double *Y_guess,
                         double *Y, double *xB) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->divJ, divJ, b);
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->eta, eta_new, b);
    memcpy(s->eta_prev, eta_old, b);
    memcpy(s->Y_n, Y_old, b);
    memcpy(s->Y, Y_guess, b);
    gp_storage_update(s, dt);
    memcpy(Y, s->Y, b);
    memcpy(xB, s->xB, b);
}
long long pfo_test_gp_eta_feasibility(pfo_state *s, double dt, int limiter, double *eta, const double *eta_old,
                                      const double *phi_new, const double *phi_old, const double *xB_old,
                                      const double *divJ) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->eta, eta, b);
    memcpy(s->eta_prev, eta_old, b);
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->xB_gp_old, xB_old, b);
    memcpy(s->divJ, divJ, b);
    const long long n = gp_eta_feasibility(s, dt, limiter);
    memcpy(eta, s->eta, b);
    return n;
}
double pfo_test_gp_sum_dy(pfo_state *s, const double *phiY, const double *etaY, const double *Y) {
    memcpy(s->Y, Y, sizeof(double) * s->N);
    return gp_sum_DY(s, phiY, etaY);
}

/* the lagged Y right-hand side (compute_Y_rhs_kernel, :2185-2266; zero mode:
 * compute_Y_rhs_sm_tangent_n_kernel, :2268-2359) from divJ, lapY and Y^n */
static void y_rhs_field(pfo_state *s, double dt, double mean_DY) {
    pfgb_params *P = &s->p;
    const int zm = P->zero_mode_enabled;
    const int gpc = gp_coupled(s);
    RLOOP_BEGIN(s)
        double Yv = s->Y[idx];
        double x = o_sigmoid_raw(Yv);
        if (x < 1e-12) x = 1e-12;
        if (x > 1.0 - 1e-12) x = 1.0 - 1e-12;
        double ld = x * (1.0 - x);
        double dYdt = s->dYdt[idx];
        double f;
        if (gpc) {  /* compute_Y_rhs_gp_kernel :2361-2430 / _conservative_ :2432-2527 */
            double han, hgn, hbn, hao, hgo, hbo;
            o_gpfrac(s->phi[idx], s->eta[idx], &han, &hgn, &hbn);
            o_gpfrac(s->phi_n[idx], s->eta_prev[idx], &hao, &hgo, &hbo);
            const double dhg = (hgn - hgo) / dt, dhb = (hbn - hbo) / dt;
            const double xs = o_sigmoid(Yv, 20.0, 1e-12);
            const double q = xs * (1.0 - xs);
            const double ss = dhg * (P->gp_xB_fixed - xs) + dhb * (1.0 - xs);
            const double hx = P->enable_Y_rhs_previous_time_level ? hao : han;
            const double gl = P->gp_y_update_mode == PFGB_GP_Y_CONSERVATIVE_RHS ? hx * q - 1.0
                                                                             : fmax(hx, P->gp_h_alpha_eps) * q - 1.0;
            const double tg = P->disable_Y_rhs_gamma_term ? 0.0 : gl * dYdt;
            const double tl = mean_DY * s->lapY[idx];
            f = s->divJ[idx] - ss - tl - tg;
        } else if (zm) {   /* compute_Y_rhs_sm_tangent_n_kernel, :2268-2359 */
            double pn = s->phi_n[idx], pp = s->phi[idx];
            double hn = o_h(pn), hpn = o_hp(pn);
            double th = hpn * ((pp - pn) / dt) * (P->v_B - x);
            double gl = (1.0 - hn) * ld - 1.0;
            f = s->divJ[idx] - th - mean_DY * s->lapY[idx] - gl * dYdt;
        } else {    /* compute_Y_rhs_kernel, :2185-2266 */
            double hn = o_h(s->phi[idx]), ho = o_h(s->phi_n[idx]);
            double dhdt = (hn - ho) / dt;
            double th = P->Y_rhs_term_h_scale * dhdt * (P->v_B - x);
            double hx = P->enable_Y_rhs_previous_time_level ? ho : hn;
            double gl = (1.0 - hx) * ld - 1.0;
            double tg = P->disable_Y_rhs_gamma_term ? 0.0 : gl * dYdt;
            f = s->divJ[idx] + (-th - mean_DY * s->lapY[idx] - tg);
        }
        s->rhs[idx] = f;
    RLOOP_END
}

/* test hooks for mu_field and y_rhs_field (the pinning tests): inputs are
 * copied into the state, outputs read back */
void pfo_test_mu(pfo_state *s, const double *Y, const double *phiY, const double *sig, double *xB, double *mu) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->Y, Y, b);
    memcpy(s->scr, phiY, b);
    for (int c = 0; c < 6; ++c)
        if (sig) memcpy(s->sig_r[c], sig + (size_t)c * s->N, b);
    mu_field(s, s->scr, s->eta);
    memcpy(xB, s->xB, b);
    memcpy(mu, s->mu, b);
}
void pfo_test_gp_y_rhs(pfo_state *s, double dt, double mean_DY, const double *divJ, const double *phi_new,
                       const double *phi_old, const double *eta_new, const double *eta_old, const double *lapY,
                       const double *Y, const double *dYdt, double *out) {
    memcpy(s->eta, eta_new, sizeof(double) * s->N);
    memcpy(s->eta_prev, eta_old, sizeof(double) * s->N);
    pfo_test_y_rhs(s, dt, mean_DY, divJ, phi_new, phi_old, lapY, Y, dYdt, out);
}
void pfo_test_y_rhs(pfo_state *s, double dt, double mean_DY, const double *divJ, const double *phi_new,
                    const double *phi_old, const double *lapY, const double *Y, const double *dYdt, double *out) {
    const size_t b = sizeof(double) * s->N;
    memcpy(s->divJ, divJ, b);
    memcpy(s->phi, phi_new, b);
    memcpy(s->phi_n, phi_old, b);
    memcpy(s->lapY, lapY, b);
    memcpy(s->Y, Y, b);
    memcpy(s->dYdt, dYdt, b);
    y_rhs_field(s, dt, mean_DY);
    memcpy(out, s->rhs, b);
}

/* divJ from the dealiased transform of mu in s->mu_k: per axis the
 * gradient, the flux J_a = M d_a mu at the mobility of phiY, etaY and x^n,
 * and the accumulated divergence (main_cuda.cu:30366-30440) */
static void divj_field(pfo_state *s, const double *phiY, const double *etaY) {
    memset(s->divJ_k, 0, sizeof(cpx) * s->Nk);
    for (int a = 0; a < 3; ++a) {
        KLOOP_BEGIN(s)   /* compute_gradient_single_component_k_kernel, :1887 */
            double ka = a == 0 ? s->kx[ii_] : (a == 1 ? s->ky[jj_] : s->kz[kk_]);
            cpx f = s->mu_k[idx];
            s->scr_k[idx].re = -ka * f.im;
            s->scr_k[idx].im = ka * f.re;
        KLOOP_END
        dealias(s, s->scr_k);
        inv(s, s->scr_k, s->scr);
        flux_field(s, phiY, etaY);
        fwd(s, s->scr, s->scr_k); dealias(s, s->scr_k);
        KLOOP_BEGIN(s)   /* divJ_accumulate_kernel, :2112 */
            double ka = a == 0 ? s->kx[ii_] : (a == 1 ? s->ky[jj_] : s->kz[kk_]);
            cpx J = s->scr_k[idx];
            s->divJ_k[idx].re += -ka * J.im;
            s->divJ_k[idx].im += ka * J.re;
        KLOOP_END
    }
    dealias(s, s->divJ_k);
    inv(s, s->divJ_k, s->divJ);
    RLOOP_BEGIN(s) s->divJ[idx] *= s->invN; RLOOP_END
}

/* ------------------------------------------------------------------ */
/* one dynamics step — main_cuda.cu:28427-31623                        */
/* ------------------------------------------------------------------ */
/* Y (composition) update and dY/dt history, main_cuda.cu:30280-30800 and
 * 31618-31623; fields at entry: phi = phi^{n+1}, phi_n = phi^n, Y = Y^n. */
static int y_update(pfo_state *s, pfgb_step_stats *st, double dt) {
    pfgb_params *P = &s->p;
    const int zm = P->zero_mode_enabled;
    const int qm = P->pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT;
    /* phi_for_Y_explicit, main_cuda.cu:30286-30291 */
    const double *phiY = zm ? s->phi_n : (qm || !P->enable_Y_rhs_previous_time_level ? s->phi : s->phi_n);
    const double *etaY = s->eta;
    const int gpc = gp_coupled(s);
    mu_field(s, phiY, etaY);
    fwd(s, s->mu, s->mu_k); dealias(s, s->mu_k);
    memcpy(s->xB_prev, s->xB, sizeof(double) * s->N);
    if (gpc) memcpy(s->xB_gp_old, s->xB, sizeof(double) * s->N);
    divj_field(s, phiY, etaY);
    if (gpc) {
        /* main_cuda.cu:30449-30503: the feasibility pass; with the local_clip
         * limiter the flux and divJ again with the limited eta, and the pass
         * once more on them.  The reference keeps x^n for the mobility in the
         * buffer of div J (d_xB_prev_r = d_divJ_r, main_cuda.cu:27858), so its
         * second flux evaluates the mobility at the first pass's div J;
         * gp_limiter_flux_from_xn = 1 takes x^n instead. */
        const int lim = P->gp_eta_mass_limiter == PFGB_GP_ETA_LIMITER_LOCAL_CLIP;
        long long nl = gp_eta_feasibility(s, dt, lim);
        if (lim) {
            if (!P->gp_limiter_flux_from_xn) memcpy(s->xB_prev, s->divJ, sizeof(double) * s->N);
            divj_field(s, phiY, etaY);
            nl += gp_eta_feasibility(s, dt, lim);
        }
        if (st) st->gp_eta_limited_cells = (int32_t)nl;
        /* eta_for_Y_explicit, main_cuda.cu:30292; global_sum_DY, :30587-30591 */
        const double *etaD = P->enable_Y_rhs_previous_time_level ? s->eta_prev : s->eta;
        const double mean_gp = gp_sum_DY(s, phiY, etaD) / (double)s->N;
        if (P->gp_y_update_mode == PFGB_GP_Y_STORAGE_EXACT || P->gp_y_update_mode == PFGB_GP_Y_PICARD_STORAGE) {
            gp_storage_update(s, dt);   /* main_cuda.cu:30927-30951 */
            RLOOP_BEGIN(s) s->dYdt[idx] = (s->Y[idx] - s->Y_n[idx]) / dt; RLOOP_END
            if (st) st->mean_DY = mean_gp;
            return PFGB_OK;
        }
        s->gp_mean_DY = mean_gp;
    }
    if (P->pf_y_update_mode == PFGB_Y_STORAGE_EXACT) {
        /* two_phase_storage_exact_Y_update_kernel, cuda_kernels.cu:2859-2921:
         * C^n + dt divJ solved for x_alpha with h^{n+1}; x^n kept where the
         * matrix storage is below its floor or the solution leaves [eps, 1-eps] */
        storage_exact_update(s, dt);
        if (st) {
            RLOOP_BEGIN(s)
                double h = o_h(phiY[idx]);
                double x = o_sigmoid_raw(s->Y_n[idx]);
                if (x < 1e-12) x = 1e-12;
                if (x > 1.0 - 1e-12) x = 1.0 - 1e-12;
                s->mass_t[idx] = o_Dmix(h, P->D_alpha, P->D_compound) * x * (1.0 - x);
            RLOOP_END
            st->mean_DY = dsum(s->mass_t, s->N) / (double)s->N;
        }
        return PFGB_OK;
    }
    if (qm) {
        /* q_transport_projection_split, main_cuda.cu:30648-30707 */
        int rc = q_transport(s, dt);
        if (st) {
            st->mean_DY = P->D_alpha * P->pf_composition_stabilizer_Dalpha_multiplier;
            st->q_redistributed_cells = s->q_redistributed;
        }
        return rc;
    }
    if (P->pf_y_update_mode == PFGB_Y_X_TRANSPORT_SPLIT) {
        /* x_transport_projection_split, main_cuda.cu:30564-30593 and
         * 30648-30676: the Laplacian of x^n, the storage source
         * compute_xB_storage_rhs_kernel (cuda_kernels.cu:2922-2951), the
         * semi-implicit update Y_semi_implicit_update_kernel (:2528-2550) with
         * the stabiliser D_alpha * multiplier in place of <DY>, then
         * xB_normalize_clamp_and_logit_kernel (:2953-2973) */
        const double mDx = P->D_alpha * P->pf_composition_stabilizer_Dalpha_multiplier;
        fwd(s, s->xB, s->divJ_k); dealias(s, s->divJ_k);   /* x^n in k space */
        KLOOP_BEGIN(s)
            double k2 = k2_at(s, ii_, jj_, kk_);
            s->Y_k[idx].re = -k2 * s->divJ_k[idx].re; s->Y_k[idx].im = -k2 * s->divJ_k[idx].im;
        KLOOP_END
        dealias(s, s->Y_k);
        inv(s, s->Y_k, s->lapY);
        xsplit_source(s, mDx);
        fwd(s, s->rhs, s->rhs_k); dealias(s, s->rhs_k);
        KLOOP_BEGIN(s)
            double den = 1.0 + dt * mDx * k2_at(s, ii_, jj_, kk_);
            cpx a = s->divJ_k[idx], r = s->rhs_k[idx];
            s->Y_k[idx].re = (a.re + dt * r.re) / den;
            s->Y_k[idx].im = (a.im + dt * r.im) / den;
        KLOOP_END
        dealias(s, s->Y_k);
        inv(s, s->Y_k, s->scr);
        xsplit_final(s, dt);
        if (st) st->mean_DY = mDx;
        return PFGB_OK;
    }
    /* Laplacian of Y, :30572-30581 */
    fwd(s, s->Y, s->Y_k); dealias(s, s->Y_k);
    KLOOP_BEGIN(s)
        double k2 = k2_at(s, ii_, jj_, kk_);
        s->Y_k[idx].re *= -k2; s->Y_k[idx].im *= -k2;
    KLOOP_END
    dealias(s, s->Y_k);
    inv(s, s->Y_k, s->lapY);
    RLOOP_BEGIN(s) s->lapY[idx] *= s->invN; RLOOP_END
    /* mean_DY, reduce_sum_DY_kernel :3870 (GP coupling: reduce_sum_DY_gp_kernel) */
    RLOOP_BEGIN(s)
        double h = o_h(phiY[idx]);
        double Dm = o_Dmix(h, P->D_alpha, P->D_compound);
        double x = o_sigmoid_raw(s->Y[idx]);
        if (x < 1e-12) x = 1e-12;
        if (x > 1.0 - 1e-12) x = 1.0 - 1e-12;
        s->mass_t[idx] = Dm * x * (1.0 - x);
    RLOOP_END
    const double mean_DY = gpc ? s->gp_mean_DY : dsum(s->mass_t, s->N) / (double)s->N;
    if (st) st->mean_DY = mean_DY;
    /* Y^n in k space (stored in divJ_k like the reference) */
    fwd(s, s->Y_n, s->divJ_k); dealias(s, s->divJ_k);
    y_rhs_field(s, dt, mean_DY);
    fwd(s, s->rhs, s->rhs_k); dealias(s, s->rhs_k);
    KLOOP_BEGIN(s)   /* Y_semi_implicit_update_kernel, :2528-2550 */
        double den = 1.0 + dt * mean_DY * k2_at(s, ii_, jj_, kk_);
        cpx a = s->divJ_k[idx], r = s->rhs_k[idx];
        s->Y_k[idx].re = (a.re + dt * r.re) / den;
        s->Y_k[idx].im = (a.im + dt * r.im) / den;
    KLOOP_END
    dealias(s, s->Y_k);
    inv(s, s->Y_k, s->Y);
    const double Ycap = P->Y_clip;
    if (zm) {
        RLOOP_BEGIN(s) s->scr[idx] = s->Y[idx] * s->invN; RLOOP_END
        int rc = zero_mode(s, s->scr, Ycap, st);
        if (rc != PFGB_OK) return rc;
    } else {
        RLOOP_BEGIN(s)   /* Y_normalize_and_clamp_kernel, :2554-2572 */
            double y = s->Y[idx] * s->invN;
            if (y > Ycap) y = Ycap;
            if (y < -P->Y_clip) y = -P->Y_clip;
            s->Y[idx] = y;
            s->xB[idx] = o_sigmoid(y, P->Y_clip, P->xB_eps);
        RLOOP_END
    }
    /* update_dY_dt_prev_kernel, :3545 */
    RLOOP_BEGIN(s) s->dYdt[idx] = (s->Y[idx] - s->Y_n[idx]) / dt; RLOOP_END
    return PFGB_OK;
}

/* new phi from its dealiased transform phi_k and the explicit drive in
 * s->rhs: phi_semi_implicit_update_kernel (cuda_kernels.cu:821-843),
 * dealias, Z2D, phi_normalize_and_clamp_kernel (:1071-1084) */
static void phi_si_update(pfo_state *s, double dt) {
    pfgb_params *P = &s->p;
    fwd(s, s->rhs, s->rhs_k); dealias(s, s->rhs_k);
    const double Ldt = P->L_phi * dt;
    KLOOP_BEGIN(s)
        double den = 1.0 + Ldt * P->kappa_phi * k2_at(s, ii_, jj_, kk_);
        cpx a = s->phi_k[idx], r = s->rhs_k[idx];
        s->phi_k[idx].re = (a.re - Ldt * r.re) / den;
        s->phi_k[idx].im = (a.im - Ldt * r.im) / den;
    KLOOP_END
    dealias(s, s->phi_k);
    inv(s, s->phi_k, s->phi);
    RLOOP_BEGIN(s)
        double v = s->phi[idx] * s->invN;
        if (v < -1e-6) v = -1e-6;
        if (v > 1.0 + 1e-6) v = 1.0 + 1e-6;
        s->phi[idx] = v;
    RLOOP_END
}

static int step_once(pfo_state *s, pfgb_step_stats *st) {
    pfgb_params *P = &s->p;
    const double dt = P->dt;
    memcpy(s->phi_n, s->phi, sizeof(double) * s->N);
    memcpy(s->eta_prev, s->eta, sizeof(double) * s->N);
    memcpy(s->Y_n, s->Y, sizeof(double) * s->N);

    const int gp_el = s->gp && P->gp_elastic_enabled;
    const int coupling = P->elastic_enabled && (!gp_el || P->gp_elastic_active_phi);
    /* conservative composition modes: the transport before the elastic solve */
    const int cons = P->pf_composition_mode != PFGB_COMPOSITION_LEGACY;
    s->cons_limited = s->cons_constrained = 0;
    if (cons) cons_transport(s);
    if (P->elastic_enabled) {
        int rc = elastic_solve(s, st);
        if (rc != PFGB_OK) return rc;
    }

    /* phi update, :29752-29860 */
    fwd(s, s->phi, s->phi_k); dealias(s, s->phi_k);
    phi_rhs(s, coupling);
    phi_si_update(s, dt);
    if (cons) {   /* the storage constraint, :29859-29880 (a rejected cell fails the step) */
        long long capped = 0;
        const long long bad = cons_constrain(s, &capped);
        s->cons_constrained = capped;
        if (st) { st->cons_limited_faces = (int)s->cons_limited; st->cons_phase_constrained = (int)capped; }
        if (bad) return PFGB_ERR_NONCONVERGED;
    }

    /* eta update (gp_zone), :29948-30006 */
    if (s->gp) {
        fwd(s, s->eta, s->eta_k); dealias(s, s->eta_k);
        eta_rhs(s);
        fwd(s, s->rhs, s->rhs_k); dealias(s, s->rhs_k);
        const double Ldt = P->gp_L_eta * dt;
        KLOOP_BEGIN(s)
            double den = 1.0 + Ldt * P->gp_kappa_eta * k2_at(s, ii_, jj_, kk_);
            cpx a = s->eta_k[idx], r = s->rhs_k[idx];
            s->eta_k[idx].re = (a.re - Ldt * r.re) / den;
            s->eta_k[idx].im = (a.im - Ldt * r.im) / den;
        KLOOP_END
        dealias(s, s->eta_k);
        inv(s, s->eta_k, s->eta);
        RLOOP_BEGIN(s)
            double v = s->eta[idx] * s->invN;
            s->eta[idx] = v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v);
        RLOOP_END
    }

    /* q split: the phase substep's storage transfer, main_cuda.cu:30241-30277 */
    s->q_rejected = 0;
    if (P->pf_y_update_mode == PFGB_Y_Q_TRANSPORT_SPLIT) q_phase(s);
    if (st) st->q_phase_rejected = s->q_rejected;

    /* the conservative modes carry the composition in their storage: no Y
     * update and no dY/dt update (main_cuda.cu:30283-30284) */
    int rc = cons ? PFGB_OK : y_update(s, st, dt);
    if (rc != PFGB_OK) return rc;
    s->step++;
    return PFGB_OK;
}

/* ------------------------------------------------------------------ */
/* minimize (mode = minimize, full model, two_phase)                    */
/* ------------------------------------------------------------------ */
/* lap = IFFT(mask (-k^2) phi_k) / N from the dealiased phi_k
 * (compute_laplacian_k_kernel, dealias, Z2D, normalize_only_kernel) */
static void phi_laplacian(pfo_state *s, double *out) {
    KLOOP_BEGIN(s)
        double k2 = k2_at(s, ii_, jj_, kk_);
        s->scr_k[idx].re = -k2 * s->phi_k[idx].re;
        s->scr_k[idx].im = -k2 * s->phi_k[idx].im;
    KLOOP_END
    dealias(s, s->scr_k);
    inv(s, s->scr_k, out);
    RLOOP_BEGIN(s) out[idx] *= s->invN; RLOOP_END
}

/* lambda = -sum h'(phi) g / sum h'(phi)^2 (compute_hprime_times_rhs_kernel,
 * compute_hprime_sq_values_kernel + gpu_reduce_sum) */
static double volume_lambda(pfo_state *s, const double *g) {
    RLOOP_BEGIN(s)
        double hp = o_hp(s->phi[idx]);
        s->mass_t[idx] = hp * g[idx];
        s->der_t[idx] = hp * hp;
    RLOOP_END
    const double shg = dsum(s->mass_t, s->N), sh2 = dsum(s->der_t, s->N);
    return fabs(sh2) > 1e-30 ? -shg / sh2 : 0.0;
}

static double mean_h_clamped(pfo_state *s) {   /* gpu_compute_vf_from_h */
    RLOOP_BEGIN(s) s->mass_t[idx] = o_h(o_clamp01(s->phi[idx])); RLOOP_END
    return dsum(s->mass_t, s->N) / (double)s->N;
}

/* V0 target when minimize_V0 <= 0: compute_effective_vf_target
 * (main_cuda.cu:2459-2490) for spherical seeds of ic_phi_seed_radius */
static double effective_vf_target(const pfgb_params *P) {
    double vf = fmin(0.999, fmax(1e-6, P->ic_vf_target_phi));
    if (!(P->ic_phi_seed_radius > 0.0)) return vf;
    const int n = P->ic_phi_num_seeds > 0 ? P->ic_phi_num_seeds : 1;
    const double R = P->ic_phi_seed_radius;
    const double Lx = P->Nx * P->dx, Ly = P->Ny * P->dy, Lz = P->Nz * P->dz;
    if (P->Ny > 2) {
        const double box = Lx * Ly * Lz;
        if (box > 0.0) vf = n * (4.0 * M_PI / 3.0) * R * R * R / box;
    } else {
        const double box = Lx * Lz;
        if (box > 0.0) vf = n * M_PI * R * R / box;
    }
    return vf;
}

/* explicit phi drive and its full variational derivative at the current
 * phi: s->rhs = g_explicit, s->mg = g_full = g_explicit - kappa Lap(phi);
 * phi_k is left holding the dealiased transform of phi */
static void phi_gradient(pfo_state *s, int coupling) {
    fwd(s, s->phi, s->phi_k); dealias(s, s->phi_k);
    if (s->p.minimize_full_model) phi_rhs(s, coupling);
    else phi_rhs_phi_only(s);   /* main_cuda.cu:29414-29429 */
    phi_laplacian(s, s->mlap);
    const double kap = s->p.kappa_phi;
    RLOOP_BEGIN(s) s->mg[idx] = s->rhs[idx] - kap * s->mlap[idx]; RLOOP_END
}

/* phi step with the volume multiplier: RHS = (g_full + kappa Lap) + lambda h'
 * (subtract_scaled_kernel with -kappa, add_volume_constraint_kernel) */
static void phi_constrained_step(pfo_state *s, double lambda, double dt) {
    const double kap = s->p.kappa_phi;
    RLOOP_BEGIN(s)
        double r = s->mg[idx] - (-kap) * s->mlap[idx];
        s->rhs[idx] = r + lambda * o_hp(s->phi[idx]);
    RLOOP_END
    phi_si_update(s, dt);
}

/* one minimize iteration, main_cuda.cu:29264-29750 (energies, phi step,
 * KKT residual), 30280-30800 (Y), 32104-32290 (post-projection, V0
 * projection), 32405-32600 (stopping rule) */
static int minimize_iter(pfo_state *s, pfgb_min_stats *ms) {
    pfgb_params *P = &s->p;
    const double dt = P->dt;   /* = minimize_dt */
    const double T = P->temperature_K, sc = P->mu_reference_scale;
    const int cv = P->thermo_convex_extrapolation_enabled;
    memcpy(s->phi_n, s->phi, sizeof(double) * s->N);
    memcpy(s->eta_prev, s->eta, sizeof(double) * s->N);
    memcpy(s->Y_n, s->Y, sizeof(double) * s->N);
    const int coupling = P->elastic_enabled;
    /* phi-only minimize (minimize_full_model = 0) carries no composition:
     * xB and Y stay zero (main_cuda.cu:27208-27217), so the eigenstrain of
     * the elastic solve and the energies is h(phi) eps00 (the phi-only
     * eigenstrain, main_cuda.cu:28816-28824 and the NULL xB of
     * :28920, :29303) */
    const int phi_only = !P->minimize_full_model;
    if (phi_only) memset(s->xB, 0, sizeof(double) * s->N);
    pfgb_step_stats st;
    memset(&st, 0, sizeof(st));
    if (P->elastic_enabled) {
        int rc = elastic_solve(s, &st);
        if (rc != PFGB_OK) return rc;
    }
    const int it = ++s->min_iter;
    elast_consts ec;
    for (int c = 0; c < 21; ++c) { ec.S[c] = rf(s, P->S[c]); ec.Sp[c] = rf(s, P->S_p[c]); }
    for (int c = 0; c < 6; ++c) { ec.e00[c] = rf(s, P->eps00[c]); ec.E0[c] = rf(s, P->E0[c]); }

    /* ---- energies (diagnostics for the CSV and the plateau test) ---- */
    double mean_h = mean_h_clamped(s);
    if (it == 1 && !(s->V0_target > 0.0))
        s->V0_target = P->ic_phi_seed_radius > 0.0 ? effective_vf_target(P) : mean_h;
    /* compute_grad_energy_density_kernel (central differences), dw energy */
    {
        const int Nx = s->Nx, Ny = s->Ny, Nz = s->Nz;
        const double kap = P->kappa_phi;
        RLOOP_BEGIN(s)
            const int k = (int)(idx % Nz);
            const size_t rem = idx / Nz;
            const int j = (int)(rem % Ny), i = (int)(rem / Ny);
            const int ip = (i + 1) % Nx, im = (i - 1 + Nx) % Nx;
            const int jp = (j + 1) % Ny, jm = (j - 1 + Ny) % Ny;
            const int kp = (k + 1) % Nz, km = (k - 1 + Nz) % Nz;
            const double *f = s->phi;
            const double gx = (f[((size_t)ip * Ny + j) * Nz + k] - f[((size_t)im * Ny + j) * Nz + k]) / (2.0 * P->dx);
            const double gy = (f[((size_t)i * Ny + jp) * Nz + k] - f[((size_t)i * Ny + jm) * Nz + k]) / (2.0 * P->dy);
            const double gz = (f[((size_t)i * Ny + j) * Nz + kp] - f[((size_t)i * Ny + j) * Nz + km]) / (2.0 * P->dz);
            s->mass_t[idx] = 0.5 * kap * (gx * gx + gy * gy + gz * gz);
            s->der_t[idx] = P->W * o_g(f[idx]);
        RLOOP_END
    }
    const double total_interface = dsum(s->mass_t, s->N) + dsum(s->der_t, s->N);
    const double F_surf = total_interface / (double)s->N;
    double F_el = 0.0, total_el_core = 0.0;
    if (P->elastic_enabled) {   /* compute_gel_density_kernel, cuda_kernels.cu:1789-1850 */
        /* the three-phase eigenstrain when GP elasticity is on (gp_zone) */
        const int gp3 = s->gp && P->gp_elastic_enabled;
        RLOOP_BEGIN(s)
            double e0[6];
            eigen_point(s, &ec, s->phi[idx], s->eta[idx], o_clamp01(s->xB[idx]), gp3, e0);
            double sd = 0.0;
            for (int c = 0; c < 6; ++c) {
                const double el = s->eps_r[c][idx] - e0[c];
                sd += (c < 3 ? 1.0 : 2.0) * s->sig_r[c][idx] * el;
            }
            s->mass_t[idx] = 0.5 * sd;
            s->der_t[idx] = 0.5 * sd * o_h(o_clamp01(s->phi[idx]));
        RLOOP_END
        F_el = dsum(s->mass_t, s->N) / (double)s->N;
        total_el_core = dsum(s->der_t, s->N);
    }
    /* compute_gbulk_excess_hat_kernel, reference state main_cuda.cu:27400-27431 */
    const double xref = P->ic_23d_xB_out;   /* > 0 (the <xB>_init fallback is not used) */
    const double g0 = (1.0 - xref) * o_muA(xref, T, sc, cv) + xref * o_muB(xref, T, sc, cv);
    RLOOP_BEGIN(s)
        const double h = o_h(o_clamp01(s->phi[idx]));
        const double x = o_clamp_eps(s->xB[idx], 1e-12);
        const double mix = (1.0 - x) * o_muA(x, T, sc, cv) + x * o_muB(x, T, sc, cv);
        s->mass_t[idx] = (1.0 - h) * mix + h * P->mu0_compound - g0;
    RLOOP_END
    /* the chemical excess and the CNT summary are full-model only
     * (main_cuda.cu:29322-29343); in phi-only minimize they stay NaN and so
     * does the total, which disables the energy-plateau test */
    const double F_chem = phi_only ? NAN : dsum(s->mass_t, s->N) / (double)s->N;
    const double F_total = phi_only ? NAN : F_chem + F_surf + F_el;
    const double muBf = o_muB(xref, T, sc, cv);
    const double F_chem_cnt = (!phi_only && mean_h > 0.0) ? mean_h * (P->mu0_compound - muBf) : NAN;
    const double F_total_cnt = phi_only ? NAN : F_surf + F_el + F_chem_cnt;
    const double F_prev = s->prev_F_total;
    s->prev_F_total = F_total;

    /* ---- phi step with the under-relaxed volume multiplier ---- */
    double eta_r = P->eta_lambda_vol;
    if (eta_r < 0.0) eta_r = 0.0;
    if (eta_r > 1.0) eta_r = 1.0;
    if (!phi_only) {
        RLOOP_BEGIN(s) s->xB[idx] = o_sigmoid(s->Y[idx], P->Y_clip, P->xB_eps); RLOOP_END   /* compute_mu_x_kernel */
    }
    phi_gradient(s, coupling);
    s->lambda_vol = (1.0 - eta_r) * s->lambda_vol + eta_r * volume_lambda(s, s->mg);
    phi_constrained_step(s, s->lambda_vol, dt);

    /* ---- projected KKT residual and rms_dphi at phi^{n+1} ---- */
    phi_gradient(s, coupling);
    {
        const double lk = volume_lambda(s, s->mg);
        RLOOP_BEGIN(s)   /* compute_projected_phi_kkt_residual_sq_kernel, :684-708 */
            const double ph = s->phi[idx];
            double r = s->mg[idx] + lk * o_hp(ph);
            if ((ph <= 1e-12 && r > 0.0) || (ph >= 1.0 - 1e-12 && r < 0.0)) r = 0.0;
            s->mass_t[idx] = r * r;
        RLOOP_END
    }
    const double rms_res = sqrt(dsum(s->mass_t, s->N) / (double)s->N);
    RLOOP_BEGIN(s) { const double d = s->phi[idx] - s->phi_n[idx]; s->mass_t[idx] = d * d; } RLOOP_END
    const double rms_dphi = sqrt(dsum(s->mass_t, s->N) / (double)s->N) / dt;

    /* ---- Y update (full model only, main_cuda.cu:30284) ---- */
    if (!phi_only) {
        int rc = y_update(s, &st, dt);
        if (rc != PFGB_OK) return rc;
    }

    /* ---- post-projection substeps, elastic frozen, eta = 1 ---- */
    for (int k = 0; k < P->minimize_post_projection_iters; ++k) {
        phi_gradient(s, coupling);
        s->lambda_vol = volume_lambda(s, s->mg);
        phi_constrained_step(s, s->lambda_vol, dt);
    }
    mean_h = mean_h_clamped(s);

    /* ---- first-order projection of <h> onto V0 ---- */
    if (s->V0_target > 1e-30 && isfinite(mean_h)) {
        const double vol_err = s->V0_target - mean_h;
        if (fabs(vol_err) > 1e-14) {
            RLOOP_BEGIN(s) { const double hp = o_hp(s->phi[idx]); s->mass_t[idx] = hp * hp; } RLOOP_END
            const double mhp2 = dsum(s->mass_t, s->N) / (double)s->N;
            const double lc = mhp2 > 1e-30 ? vol_err / mhp2 : 0.0;
            RLOOP_BEGIN(s)   /* apply_volume_projection_kernel, :636-645 */
                const double ph = s->phi[idx];
                s->phi[idx] = o_clamp01(ph + lc * o_hp(ph));
            RLOOP_END
            mean_h = mean_h_clamped(s);
        }
    }

    /* ---- stopping rule ---- */
    double edr = NAN;
    if (isfinite(F_prev) && isfinite(F_total)) edr = fabs(F_total - F_prev) / fmax(fabs(F_prev), 1e-20);
    const double ver = s->V0_target > 1e-30 ? fabs(mean_h - s->V0_target) / (s->V0_target + 1e-30) : 0.0;
    /* rms_dY is a full-model column (NaN in phi-only minimize, :32425-32440) */
    double rms_dY = NAN;
    if (!phi_only) {
        RLOOP_BEGIN(s) { const double d = s->Y[idx] - s->Y_n[idx]; s->mass_t[idx] = d * d; } RLOOP_END
        rms_dY = sqrt(dsum(s->mass_t, s->N) / (double)s->N) / dt;
    }
    const int vol_ok = isfinite(ver) && ver < P->minimize_vol_err_rel_threshold;
    const int res_ok = isfinite(rms_res) && rms_res < P->minimize_rms_res_threshold;
    int condA, condB;
    if (phi_only) {   /* :32541-32550: phi convergence and the energy plateau */
        condA = isfinite(rms_dphi) && rms_dphi < P->minimize_rms_dphi_threshold && res_ok && vol_ok;
        condB = isfinite(edr) && edr < P->minimize_energy_diff_rel_threshold && isfinite(rms_dphi) &&
                rms_dphi < 5.0 * P->minimize_rms_dphi_threshold && res_ok && vol_ok;
    } else {
        condA = isfinite(rms_dphi) && isfinite(rms_dY) && rms_dphi < P->minimize_rms_dphi_threshold &&
                rms_dY < P->minimize_rms_dY_threshold && res_ok && vol_ok;
        condB = isfinite(edr) && edr < P->minimize_energy_diff_rel_threshold && isfinite(rms_dphi) &&
                isfinite(rms_dY) && rms_dphi < 5.0 * P->minimize_rms_dphi_threshold &&
                rms_dY < 5.0 * P->minimize_rms_dY_threshold && res_ok && vol_ok;
    }
    const double pt = (double)it * dt;
    const int pt_ok = isfinite(pt) && pt + 1e-14 >= P->minimize_min_pseudo_time;
    s->conv_count = ((condA || condB) && pt_ok) ? s->conv_count + 1 : 0;
    if (s->conv_count >= P->minimize_convergence_steps && !s->converged_iter) s->converged_iter = it;

    /* ---- xB safety clamp of the monitor step (every iteration here;
     *      full model only, main_cuda.cu:25262) ---- */
    double xmax = -1e300;
    for (size_t i = 0; i < s->N; ++i) if (s->xB[i] > xmax) xmax = s->xB[i];
    int clamped = 0;
    if (!phi_only && xmax > P->minimize_xB_max_safe + 1e-12) {   /* launch_clamp_xB_max_kernel */
        clamped = 1;
        RLOOP_BEGIN(s) if (s->xB[idx] > P->minimize_xB_max_safe) s->xB[idx] = P->minimize_xB_max_safe; RLOOP_END
    }
    s->step++;
    if (ms) {
        ms->iteration = it;
        ms->converged = s->converged_iter != 0;
        ms->converged_iteration = s->converged_iter;
        ms->convergence_count = s->conv_count;
        ms->condA = condA; ms->condB = condB;
        ms->xB_clamped = clamped;
        ms->elastic_iterations = st.elastic_iterations;
        ms->elastic_relative_residual = st.elastic_relative_residual;
        ms->mean_h = mean_h; ms->V0_target = s->V0_target; ms->lambda_vol = s->lambda_vol;
        ms->F_surf = F_surf; ms->F_el = F_el; ms->F_chem_excess = F_chem; ms->F_total_excess = F_total;
        ms->F_chem_CNT = F_chem_cnt; ms->F_total_CNT = F_total_cnt;
        ms->total_interface_sum = total_interface; ms->total_el_core_sum = total_el_core;
        ms->rms_res = rms_res; ms->rms_dphi = rms_dphi; ms->rms_dY = rms_dY;
        ms->energy_diff_rel = edr; ms->vol_err_rel = ver;
    }
    return PFGB_OK;
}

int pfo_minimize(pfo_state *s, int max_iter, int stop_on_convergence, pfgb_min_stats *ms) {
    const pfgb_params *P = &s->p;
    /* gp_zone minimize: the same iteration with eta held fixed (eta evolves
     * in dynamics only, main_cuda.cu:29948-30006) and the GP forms of the
     * phi drive, the mu of the flux and the eigenstrain */
    if (P->mode != PFGB_MODE_MINIMIZE || P->zero_mode_enabled || (s->gp && !P->minimize_full_model))
        return PFGB_ERR_UNSUPPORTED;
    for (int i = 0; i < max_iter; ++i) {
        int rc = minimize_iter(s, ms);
        if (rc != PFGB_OK) return rc;
        if (stop_on_convergence && s->converged_iter) break;
    }
    return PFGB_OK;
}

int pfo_load_fields(pfo_state *s, const double *phi, const double *xB, const double *eta,
                    const double *dYdt) {
    const pfgb_params *P = &s->p;
    memcpy(s->phi, phi, sizeof(double) * s->N);
    memcpy(s->xB, xB, sizeof(double) * s->N);
    if (eta) memcpy(s->eta, eta, sizeof(double) * s->N); else memset(s->eta, 0, sizeof(double) * s->N);
    if (dYdt) memcpy(s->dYdt, dYdt, sizeof(double) * s->N); else memset(s->dYdt, 0, sizeof(double) * s->N);
    for (size_t i = 0; i < s->N; ++i) s->Y[i] = o_logit(s->xB[i], P->xB_eps, P->Y_clip);
    s->warm_valid = 0;
    s->warm_count = 0;
    s->step = 0;
    /* gpu_reduce_sum_xBtot, main_cuda.cu:28079-28086 */
    RLOOP_BEGIN(s)
        double h = o_h(s->phi[idx]);
        s->mass_t[idx] = (1.0 - h) * s->xB[idx] + P->v_B * h;
    RLOOP_END
    s->target_mass = dsum(s->mass_t, s->N);
    q_from_phi_xB(s);   /* initialize_q_alpha_kernel, main_cuda.cu:28051-28053 */
    cons_init(s);       /* initialize_conservative_storage_kernel, main_cuda.cu:28054-28058 */
    for (int c = 0; c < 6; ++c) {
        memset(s->sig_r[c], 0, sizeof(double) * s->N);
        memset(s->eps_r[c], 0, sizeof(double) * s->N);
    }
    return PFGB_OK;
}

int pfo_step(pfo_state *s, int nsteps, pfgb_step_stats *st) {
    if (st) memset(st, 0, sizeof(*st));
    for (int i = 0; i < nsteps; ++i) {
        int rc = step_once(s, st);
        if (rc != PFGB_OK) return rc;
    }
    if (st) st->step = s->step;
    return PFGB_OK;
}

int pfo_read_fields(const pfo_state *s, double *phi, double *xB, double *Y, double *eta,
                    double *dYdt) {
    const size_t b = sizeof(double) * s->N;
    if (phi) memcpy(phi, s->phi, b);
    if (xB) memcpy(xB, s->xB, b);
    if (Y) memcpy(Y, s->Y, b);
    if (eta) memcpy(eta, s->eta, b);
    if (dYdt) memcpy(dYdt, s->dYdt, b);
    return PFGB_OK;
}

int pfo_read_elastic(const pfo_state *s, double *sigma6, double *strain6) {
    for (int c = 0; c < 6; ++c) {
        if (sigma6) memcpy(sigma6 + (size_t)c * s->N, s->sig_r[c], sizeof(double) * s->N);
        if (strain6) memcpy(strain6 + (size_t)c * s->N, s->eps_r[c], sizeof(double) * s->N);
    }
    return PFGB_OK;
}

int pfo_read_displacement_k(const pfo_state *s, double *u3) {
    for (int c = 0; c < 3; ++c) memcpy(u3 + (size_t)c * 2 * s->Nk, s->u_k[c], sizeof(cpx) * s->Nk);
    return PFGB_OK;
}

int pfo_diagnostics(const pfo_state *s, pfgb_diag *d) {
    const pfgb_params *P = &s->p;
    double *t = (double *)malloc(sizeof(double) * s->N);
    double *u = (double *)malloc(sizeof(double) * s->N);
    double *w = (double *)malloc(sizeof(double) * s->N);
    double *f = (double *)malloc(sizeof(double) * s->N);
    double pmin = 1e300, pmax = -1e300, xmin = 1e300, xmax = -1e300;
    for (size_t i = 0; i < s->N; ++i) {
        double h = o_h(o_clamp01(s->phi[i]));
        t[i] = h;
        double hh = o_h(s->phi[i]);
        if (gp_coupled(s)) {   /* reduce_sum_xBtot_gp_kernel, cuda_kernels.cu:3830-3860 */
            double ha, hg, hb;
            o_gpfrac(s->phi[i], s->eta[i], &ha, &hg, &hb);
            u[i] = ha * s->xB[i] + hg * P->gp_xB_fixed + hb;
        } else {
            u[i] = (1.0 - hh) * s->xB[i] + P->v_B * hh;
        }
        /* reduce_sum_N_in_N_if_kernel, cuda_kernels.cu:3746-3786 */
        w[i] = s->phi[i] > 0.5 ? 1.0 : 0.0;
        f[i] = (s->phi[i] > 0.12 && s->phi[i] < 0.88) ? 1.0 : 0.0;
        if (s->phi[i] < pmin) pmin = s->phi[i];
        if (s->phi[i] > pmax) pmax = s->phi[i];
        if (s->xB[i] < xmin) xmin = s->xB[i];
        if (s->xB[i] > xmax) xmax = s->xB[i];
    }
    d->vf_precip = dsum(t, s->N) / (double)s->N;
    d->mass_xBtot = dsum(u, s->N);
    d->mean_xB = dsum(s->xB, s->N) / (double)s->N;
    d->n_in = dsum(w, s->N);
    d->n_if = dsum(f, s->N);
    d->phi_min = pmin; d->phi_max = pmax; d->xB_min = xmin; d->xB_max = xmax;
    free(t); free(u); free(w); free(f);
    return PFGB_OK;
}

/* Spectral bounds of the increment operator -Gamma0 (h dC) for h in [0, 1]:
 * [min(0, -mu_max), max(0, -mu_min)] with mu the generalised eigenvalues of
 * (dC, C0) in Voigt form (engineering shear), widened by 2% of the length.
 * Restated here with a symmetric C0^(-1/2) built from C0's own eigen
 * decomposition (Jacobi), then Jacobi on C0^(-1/2) dC C0^(-1/2). */
static void o_jacobi6(double A[6][6], double V[6][6]) {
    for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) V[i][j] = (i == j);
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int i = 0; i < 6; ++i) for (int j = i + 1; j < 6; ++j) off += A[i][j] * A[i][j];
        if (off < 1e-40) break;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) {
                if (fabs(A[p][q]) < 1e-300) continue;
                const double phi = 0.5 * atan2(2.0 * A[p][q], A[q][q] - A[p][p]);
                const double c = cos(phi), sn = sin(phi);
                for (int k = 0; k < 6; ++k) {   /* columns p, q */
                    const double ap = A[k][p], aq = A[k][q];
                    A[k][p] = c * ap - sn * aq;
                    A[k][q] = sn * ap + c * aq;
                }
                for (int k = 0; k < 6; ++k) {   /* rows p, q */
                    const double ap = A[p][k], aq = A[q][k];
                    A[p][k] = c * ap - sn * aq;
                    A[q][k] = sn * ap + c * aq;
                }
                for (int k = 0; k < 6; ++k) {
                    const double vp = V[k][p], vq = V[k][q];
                    V[k][p] = c * vp - sn * vq;
                    V[k][q] = sn * vp + c * vq;
                }
            }
    }
}

int pfo_chebyshev_bounds(const double S[21], const double Sp[21], double *a, double *b) {
    static const int st[6] = {0, 6, 11, 15, 18, 20};
    double C[6][6], D[6][6], V[6][6], W[6][6], T[6][6], B[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            C[i][j] = S[st[lo] + hi - lo];
            D[i][j] = Sp[st[lo] + hi - lo];
        }
    o_jacobi6(C, V);   /* C0 = V diag V^T */
    for (int i = 0; i < 6; ++i) if (!(C[i][i] > 0.0)) return 0;
    for (int i = 0; i < 6; ++i)   /* W = C0^(-1/2) = V diag(1/sqrt) V^T */
        for (int j = 0; j < 6; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += V[i][k] * V[j][k] / sqrt(C[k][k]);
            W[i][j] = t;
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += D[i][k] * W[k][j];
            T[i][j] = t;
        }
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double t = 0.0;
            for (int k = 0; k < 6; ++k) t += W[i][k] * T[k][j];
            B[i][j] = t;
        }
    o_jacobi6(B, V);
    double mn = B[0][0], mx = B[0][0];
    for (int i = 1; i < 6; ++i) { if (B[i][i] < mn) mn = B[i][i]; if (B[i][i] > mx) mx = B[i][i]; }
    double lo = fmin(0.0, -mx), hi = fmax(0.0, -mn);
    const double w = 0.02 * (hi - lo);
    lo -= w;
    hi += w;
    if (!isfinite(lo) || !isfinite(hi) || !(hi < 1.0)) return 0;
    *a = lo;
    *b = hi;
    return 1;
}

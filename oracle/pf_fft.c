/*
 * pf_fft.c — FP64 mixed-radix FFT for the CPU oracle (test infrastructure).
 *
 * Stands in for the cuFFT calls of the reference (main_cuda.cu:28163-28173:
 * cufftPlan3d D2Z/Z2D and R2C/C2R over the [Nx][Ny][Nz] C-order grid, half
 * spectrum along z).  cuFFT computes the plain DFT
 *     X[m] = sum_n x[n] exp(-2 pi i m n / N)   (forward, unnormalised)
 * and its inverse with exp(+...), also unnormalised; that is all this file
 * restates.  Algorithm: Stockham autosort, radices 2/3/4/5 coded directly,
 * any other prime factor (41 at N=246) as a direct DFT stage.  Twiddles are
 * read from a per-length table of exp(-2 pi i m / n) built in FP64.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cpx;

typedef struct {
    int n;
    int nstage;
    int radix[40];
    cpx *w;        /* w[m] = exp(-2 pi i m / n) */
} plan1d;

static void plan_init(plan1d *p, int n) {
    p->n = n;
    p->nstage = 0;
    int m = n;
    while (m > 1 && m % 4 == 0) { p->radix[p->nstage++] = 4; m /= 4; }
    while (m > 1 && m % 2 == 0) { p->radix[p->nstage++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { p->radix[p->nstage++] = f; m /= f; }
    }
    p->w = (cpx *)malloc(sizeof(cpx) * (size_t)(n > 0 ? n : 1));
    const double two_pi = 6.283185307179586476925286766559;
    for (int k = 0; k < n; ++k) {
        double a = two_pi * (double)k / (double)n;
        p->w[k].re = cos(a);
        p->w[k].im = -sin(a);
    }
}

static void plan_free(plan1d *p) { free(p->w); p->w = NULL; }

/* one length-n transform; x is overwritten, tmp has n entries */
static void fft_exec(const plan1d *p, int sign, cpx *x, cpx *tmp) {
    const int n = p->n;
    if (n <= 1) return;
    cpx *src = x, *dst = tmp;
    int Ns = 1;
    for (int s = 0; s < p->nstage; ++s) {
        const int R = p->radix[s];
        const int nb = n / R;
        const int wstep = n / (Ns * R);       /* W_{Ns R} = W_n^{wstep} */
        for (int j = 0; j < nb; ++j) {
            const int k = j % Ns;
            cpx v[64];
            cpx *vb = v;
            cpx *heap = NULL;
            if (R > 64) { heap = (cpx *)malloc(sizeof(cpx) * (size_t)R); vb = heap; }
            for (int r = 0; r < R; ++r) {
                cpx a = src[j + r * nb];
                int e = (int)(((long long)r * k * wstep) % n);
                cpx w = p->w[e];
                if (sign > 0) w.im = -w.im;
                vb[r].re = a.re * w.re - a.im * w.im;
                vb[r].im = a.re * w.im + a.im * w.re;
            }
            const int base = (j / Ns) * Ns * R + k;
            if (R == 2) {
                cpx a = vb[0], b = vb[1];
                dst[base].re = a.re + b.re;      dst[base].im = a.im + b.im;
                dst[base + Ns].re = a.re - b.re; dst[base + Ns].im = a.im - b.im;
            } else if (R == 4) {
                cpx a0 = vb[0], a1 = vb[1], a2 = vb[2], a3 = vb[3];
                cpx t0 = {a0.re + a2.re, a0.im + a2.im};
                cpx t1 = {a0.re - a2.re, a0.im - a2.im};
                cpx t2 = {a1.re + a3.re, a1.im + a3.im};
                cpx t3 = {a1.re - a3.re, a1.im - a3.im};
                /* -i*t3 for forward, +i*t3 for inverse */
                cpx t3r = (sign < 0) ? (cpx){t3.im, -t3.re} : (cpx){-t3.im, t3.re};
                dst[base].re = t0.re + t2.re;           dst[base].im = t0.im + t2.im;
                dst[base + Ns].re = t1.re + t3r.re;     dst[base + Ns].im = t1.im + t3r.im;
                dst[base + 2 * Ns].re = t0.re - t2.re;  dst[base + 2 * Ns].im = t0.im - t2.im;
                dst[base + 3 * Ns].re = t1.re - t3r.re; dst[base + 3 * Ns].im = t1.im - t3r.im;
            } else {
                /* direct DFT of length R: out[q] = sum_r v[r] W_R^{rq} */
                const int wr = n / R;
                for (int q = 0; q < R; ++q) {
                    double sr = 0.0, si = 0.0;
                    for (int r = 0; r < R; ++r) {
                        int e = (int)(((long long)r * q) % R) * wr;
                        cpx w = p->w[e];
                        if (sign > 0) w.im = -w.im;
                        sr += vb[r].re * w.re - vb[r].im * w.im;
                        si += vb[r].re * w.im + vb[r].im * w.re;
                    }
                    dst[base + q * Ns].re = sr;
                    dst[base + q * Ns].im = si;
                }
            }
            if (heap) free(heap);
        }
        cpx *t = src; src = dst; dst = t;
        Ns *= R;
    }
    if (src != x) memcpy(x, src, sizeof(cpx) * (size_t)n);
}

void pfo_fft1d(int n, int sign, const double *in, double *out) {
    plan1d p;
    plan_init(&p, n);
    cpx *x = (cpx *)malloc(sizeof(cpx) * (size_t)n);
    cpx *t = (cpx *)malloc(sizeof(cpx) * (size_t)n);
    memcpy(x, in, sizeof(cpx) * (size_t)n);
    fft_exec(&p, sign, x, t);
    memcpy(out, x, sizeof(cpx) * (size_t)n);
    free(x); free(t);
    plan_free(&p);
}

/* complex transforms along y then x of a [Nx][Ny][NzC] array, in place */
static void fft_xy(int Nx, int Ny, int NzC, int sign, cpx *a,
                   const plan1d *py, const plan1d *px) {
    const int maxn = (Nx > Ny ? Nx : Ny);
#pragma omp parallel
    {
        cpx *line = (cpx *)malloc(sizeof(cpx) * (size_t)maxn);
        cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)maxn);
        /* y axis: fixed (i,k), stride NzC */
#pragma omp for schedule(static)
        for (long long ik = 0; ik < (long long)Nx * NzC; ++ik) {
            const int i = (int)(ik / NzC), k = (int)(ik % NzC);
            cpx *base = a + (size_t)i * Ny * NzC + k;
            for (int j = 0; j < Ny; ++j) line[j] = base[(size_t)j * NzC];
            fft_exec(py, sign, line, tmp);
            for (int j = 0; j < Ny; ++j) base[(size_t)j * NzC] = line[j];
        }
        /* x axis: fixed (j,k), stride Ny*NzC */
#pragma omp for schedule(static)
        for (long long jk = 0; jk < (long long)Ny * NzC; ++jk) {
            cpx *base = a + jk;
            const size_t st = (size_t)Ny * NzC;
            for (int i = 0; i < Nx; ++i) line[i] = base[(size_t)i * st];
            fft_exec(px, sign, line, tmp);
            for (int i = 0; i < Nx; ++i) base[(size_t)i * st] = line[i];
        }
        free(line); free(tmp);
    }
}

void pfo_fft3d_r2c(int Nx, int Ny, int Nz, const double *in, double *out) {
    const int NzC = Nz / 2 + 1;
    plan1d pz, py, px;
    plan_init(&pz, Nz); plan_init(&py, Ny); plan_init(&px, Nx);
    cpx *o = (cpx *)out;
#pragma omp parallel
    {
        cpx *line = (cpx *)malloc(sizeof(cpx) * (size_t)Nz);
        cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)Nz);
#pragma omp for schedule(static)
        for (long long ij = 0; ij < (long long)Nx * Ny; ++ij) {
            const double *row = in + (size_t)ij * Nz;
            for (int k = 0; k < Nz; ++k) { line[k].re = row[k]; line[k].im = 0.0; }
            fft_exec(&pz, -1, line, tmp);
            memcpy(o + (size_t)ij * NzC, line, sizeof(cpx) * (size_t)NzC);
        }
        free(line); free(tmp);
    }
    fft_xy(Nx, Ny, NzC, -1, o, &py, &px);
    plan_free(&pz); plan_free(&py); plan_free(&px);
}

void pfo_fft3d_c2r(int Nx, int Ny, int Nz, const double *in, double *out) {
    const int NzC = Nz / 2 + 1;
    plan1d pz, py, px;
    plan_init(&pz, Nz); plan_init(&py, Ny); plan_init(&px, Nx);
    const size_t nk = (size_t)Nx * Ny * NzC;
    cpx *a = (cpx *)malloc(sizeof(cpx) * nk);
    memcpy(a, in, sizeof(cpx) * nk);
    fft_xy(Nx, Ny, NzC, +1, a, &py, &px);
#pragma omp parallel
    {
        cpx *line = (cpx *)malloc(sizeof(cpx) * (size_t)Nz);
        cpx *tmp = (cpx *)malloc(sizeof(cpx) * (size_t)Nz);
#pragma omp for schedule(static)
        for (long long ij = 0; ij < (long long)Nx * Ny; ++ij) {
            const cpx *h = a + (size_t)ij * NzC;
            /* Hermitian extension along z; the real part of the inverse
             * ignores the imaginary parts of the k=0 / Nyquist bins. */
            for (int k = 0; k < NzC; ++k) line[k] = h[k];
            for (int k = NzC; k < Nz; ++k) {
                line[k].re = h[Nz - k].re;
                line[k].im = -h[Nz - k].im;
            }
            fft_exec(&pz, +1, line, tmp);
            double *row = out + (size_t)ij * Nz;
            for (int k = 0; k < Nz; ++k) row[k] = line[k].re;
        }
        free(line); free(tmp);
    }
    free(a);
    plan_free(&pz); plan_free(&py); plan_free(&px);
}

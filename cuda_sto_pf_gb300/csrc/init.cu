// init.cu — seeded initial fields on the device (initialize_fields_cuda,
// main_cuda.cu:15157-15430), for runs started without raw fields.
//
//  1. radius R: ic_phi_seed_radius when > 0, else the radius at which
//     N seeds fill ic_vf_init_phi of the box; axes (Rx, Ry, Rz) from the
//     shape mode and axis ratios, normalised to the volume (area in 2-D) of
//     the radius-R sphere (compute_seed_axes_from_radius, :2430-2457);
//  2. centres: one seed at the box centre, several placed by srand(seed) /
//     rand() inside a margin (generate_seed_centers_uniform, :2335-2383),
//     each shifted by init_center_shift (periodically wrapped);
//  3. phi = max over seeds of 1/2 (1 + tanh((1 - r_eff) min_axis / w)),
//     r_eff the ellipsoidal radius in the seed frame (rows of the tilt
//     rotation, build_seed_rotation_from_normal :15627-15675), periodic
//     distances; then uniform noise phi <- clamp01(phi + a (2u - 1)) with u
//     from a per-cell 64-bit hash (init_phi_kernel :2244-2312,
//     apply_phi_noise_kernel :2386-2406);
//  4. xB = clamp_eps((1 - h) xB_out + h xB_eq), xB_out = ic_23d_xB_out when
//     > 0, else solved from the diffuse-interface lever rule with <h> and
//     <h^2> (:15316-15356, init_xB_Y_from_phi_kernel :2314-2333).
// The steps and constants are the reference's, so the same parameters give
// the same initial state; the code is this library's (the reductions of
// <h>, <h^2> run on the device in float64).
#include <cmath>
#include <cstdlib>
#include <vector>

#include "common.cuh"

namespace {

__device__ __forceinline__ double periodic_d(double x, double c, double L) {
    double d = x - c;
    if (d > 0.5 * L) d -= L;
    if (d < -0.5 * L) d += L;
    return d;
}

struct SeedGeom {
    int Nx, Ny, Nz, nseeds, rotate, is3d;
    double dx, dy, dz, Lx, Ly, Lz, w, Rx, Ry, Rz, min_axis;
};

__global__ void k_seed_phi(SeedGeom g, const double *__restrict__ centers, const double *__restrict__ rot,
                           double *__restrict__ phi, double noise_amp, unsigned long long noise_seed) {
    const long long N = (long long)g.Nx * g.Ny * g.Nz;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < N;
         idx += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(idx / ((long long)g.Ny * g.Nz));
        const long long rem = idx - (long long)i * g.Ny * g.Nz;
        const int j = (int)(rem / g.Nz), k = (int)(rem - (long long)j * g.Nz);
        const double x = i * g.dx, y = j * g.dy, z = k * g.dz;
        double best = 0.0;
        for (int s = 0; s < g.nseeds; ++s) {
            const double rx = periodic_d(x, centers[3 * s], g.Lx);
            const double ry = g.is3d ? periodic_d(y, centers[3 * s + 1], g.Ly) : 0.0;
            const double rz = periodic_d(z, centers[3 * s + 2], g.Lz);
            double qx = rx, qy = ry, qz = rz;
            if (g.rotate) {   // q = R r with the rows of R the seed frame
                const double *R = rot + 9 * s;
                qx = R[0] * rx + R[1] * ry + R[2] * rz;
                qy = R[3] * rx + R[4] * ry + R[5] * rz;
                qz = R[6] * rx + R[7] * ry + R[8] * rz;
            }
            double r2 = qx * qx / (g.Rx * g.Rx) + qz * qz / (g.Rz * g.Rz);
            if (g.is3d) r2 += qy * qy / (g.Ry * g.Ry);
            const double seed = 0.5 * (1.0 + tanh((1.0 - sqrt(r2)) * (g.min_axis / g.w)));
            best = seed > best ? seed : best;
        }
        double p = clamp01(best);
        if (noise_amp > 0.0) {
            // per-cell 64-bit hash (apply_phi_noise_kernel): multiply-xorshift
            // finaliser of seed ^ (idx + 1) * golden-ratio-like constant
            unsigned long long h = noise_seed ^ (unsigned long long)(idx + 1) * 2862933555777941757ULL;
            h ^= h >> 33;
            h *= 0xff51afd7ed558ccdULL;
            h ^= h >> 33;
            h *= 0xc4ceb9fe1a85ec53ULL;
            h ^= h >> 33;
            const double u = (double)(h & 0xFFFFFFFFULL) / (double)0xFFFFFFFFULL;
            p = clamp01(p + (2.0 * u - 1.0) * noise_amp);
        }
        phi[idx] = p;
    }
}

// block partials of sum h, sum h^2 (float64, fixed order inside the block)
__global__ void k_h_moments(const double *__restrict__ phi, long long N, double *__restrict__ part) {
    __shared__ double s1[256], s2[256];
    double a = 0.0, b = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const double h = pf_h(phi[i]);
        a += h;
        b += h * h;
    }
    s1[threadIdx.x] = a;
    s2[threadIdx.x] = b;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s1[threadIdx.x] += s1[threadIdx.x + w];
            s2[threadIdx.x] += s2[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = s1[0];
        part[2 * blockIdx.x + 1] = s2[0];
    }
}

__global__ void k_seed_xB(const double *__restrict__ phi, double *__restrict__ xB, long long N, double xB_out,
                          double xB_eq, double eps) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        const double h = pf_h(clamp01(phi[i]));
        xB[i] = clamp_eps((1.0 - h) * xB_out + h * xB_eq, eps);
    }
}

// rows e1, e2, n of the frame whose third axis is the tilted normal
void tilt_frame(double theta_deg, double phi_deg, double R[9]) {
    const double d2r = PFGB_PI / 180.0;
    double nx = std::sin(theta_deg * d2r) * std::cos(phi_deg * d2r);
    double ny = std::sin(theta_deg * d2r) * std::sin(phi_deg * d2r);
    double nz = std::cos(theta_deg * d2r);
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    const double nn = std::sqrt(nx * nx + ny * ny + nz * nz);
    if (nn < 1e-8) { for (int k = 0; k < 9; ++k) R[k] = I[k]; return; }
    nx /= nn; ny /= nn; nz /= nn;
    // reference vector not parallel to n: z, or y when n is close to z
    const double rx = 0.0, ry = std::fabs(nz) > 0.9 ? 1.0 : 0.0, rz = std::fabs(nz) > 0.9 ? 0.0 : 1.0;
    double e1x = ry * nz - rz * ny, e1y = rz * nx - rx * nz, e1z = rx * ny - ry * nx;
    const double en = std::sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    if (en < 1e-12) { for (int k = 0; k < 9; ++k) R[k] = I[k]; return; }
    e1x /= en; e1y /= en; e1z /= en;
    const double e2x = ny * e1z - nz * e1y, e2y = nz * e1x - nx * e1z, e2z = nx * e1y - ny * e1x;
    const double out[9] = {e1x, e1y, e1z, e2x, e2y, e2z, nx, ny, nz};
    for (int k = 0; k < 9; ++k) R[k] = out[k];
}

void seed_axes(const pfgb_params &P, double R, bool is3d, double *Rx, double *Ry, double *Rz) {
    if (P.init_shape_mode <= 0) { *Rx = *Ry = *Rz = R; return; }
    const double ax = P.init_axis_ratio_rx > 0.0 ? P.init_axis_ratio_rx : 1.0;
    const double ay = P.init_axis_ratio_ry > 0.0 ? P.init_axis_ratio_ry : 1.0;
    const double az = P.init_axis_ratio_rz > 0.0 ? P.init_axis_ratio_rz : 1.0;
    if (is3d) {
        double sc = std::cbrt(ax * ay * az);
        if (!(sc > 0.0)) sc = 1.0;
        *Rx = R * ax / sc; *Ry = R * ay / sc; *Rz = R * az / sc;
    } else {
        double sc = std::sqrt(ax * az);
        if (!(sc > 0.0)) sc = 1.0;
        *Rx = R * ax / sc; *Ry = R; *Rz = R * az / sc;
    }
}

// centres: the box centre for one seed; otherwise srand(seed) / rand()
// inside [margin, L - margin] (2-D: y at the mid plane)
std::vector<double> seed_centres(const pfgb_params &P) {
    const int n = P.ic_phi_num_seeds > 0 ? P.ic_phi_num_seeds : 1;
    const double Lx = P.Nx * P.dx, Ly = P.Ny * P.dy, Lz = P.Nz * P.dz;
    std::vector<double> c(3 * (size_t)n);
    if (n == 1) {
        c[0] = 0.5 * Lx; c[1] = 0.5 * Ly; c[2] = 0.5 * Lz;
    } else {
        const double w = P.ic_phi_iface_w > 0.0 ? P.ic_phi_iface_w * P.dx : P.dx;
        const double Rest = P.ic_phi_seed_radius > 0.0 ? P.ic_phi_seed_radius : 10.0 * P.dx;
        const double m = Rest + 2.0 * w;
        const double mx = std::fmin(m, 0.1 * Lx), my = std::fmin(m, 0.1 * Ly), mz = std::fmin(m, 0.1 * Lz);
        srand((unsigned int)P.seed);
        for (int s = 0; s < n; ++s) {
            const double ux = (double)rand() / (double)RAND_MAX;
            const double uy = P.Ny > 2 ? (double)rand() / (double)RAND_MAX : 0.0;
            const double uz = (double)rand() / (double)RAND_MAX;
            c[3 * s] = mx + ux * (Lx - 2.0 * mx);
            c[3 * s + 1] = P.Ny > 2 ? my + uy * (Ly - 2.0 * my) : 0.5 * Ly;
            c[3 * s + 2] = mz + uz * (Lz - 2.0 * mz);
        }
    }
    const double sh[3] = {P.init_center_shift_x, P.init_center_shift_y, P.init_center_shift_z};
    const double L[3] = {Lx, Ly, Lz};
    if (sh[0] != 0.0 || sh[1] != 0.0 || sh[2] != 0.0)
        for (int s = 0; s < n; ++s)
            for (int a = 0; a < 3; ++a) {
                double v = c[3 * s + a] + sh[a];
                if (v < 0.0) v += L[a];
                if (v >= L[a]) v -= L[a];
                c[3 * s + a] = v;
            }
    return c;
}

double vf_target(const pfgb_params &P) {   // compute_effective_vf_target, :2459-2490
    const int n = P.ic_phi_num_seeds > 0 ? P.ic_phi_num_seeds : 1;
    const bool is3d = P.Ny > 2;
    const double Lx = P.Nx * P.dx, Ly = P.Ny * P.dy, Lz = P.Nz * P.dz;
    double vf = std::fmin(0.999, std::fmax(1e-6, P.ic_vf_target_phi));
    if (!(P.ic_phi_seed_radius > 0.0)) return vf;
    double Rx, Ry, Rz;
    seed_axes(P, P.ic_phi_seed_radius, is3d, &Rx, &Ry, &Rz);
    if (is3d) { if (Lx * Ly * Lz > 0.0) vf = n * (4.0 * PFGB_PI / 3.0) * Rx * Ry * Rz / (Lx * Ly * Lz); }
    else if (Lx * Lz > 0.0) vf = n * PFGB_PI * Rx * Rz / (Lx * Lz);
    return std::fmin(0.999, std::fmax(1e-6, vf));
}

#define INIT_TRY(x)                                                                               \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            pfgb_set_error_msg("seeded fields: %s failed: %s", #x, cudaGetErrorString(e_));       \
            return PFGB_ERR_CUDA;                                                                 \
        }                                                                                         \
    } while (0)

}  // namespace

// phi and xB (float64) of the seeded initial state into device buffers;
// scratch holds 2 * 304 doubles
pfgb_status pfgb_seed_fields_device(const pfgb_params *pp, double *d_phi, double *d_xB, double *d_scratch,
                                    cudaStream_t stream) {
    const pfgb_params &P = *pp;
    if (!(P.dx > 0.0 && P.dy > 0.0 && P.dz > 0.0) || P.Nx < 1 || P.Ny < 1 || P.Nz < 1) {
        pfgb_set_error_msg("seeded fields: invalid grid");
        return PFGB_ERR_INVALID;
    }
    const bool is3d = P.Ny > 2;
    const int n = P.ic_phi_num_seeds > 0 ? P.ic_phi_num_seeds : 1;
    const double Lx = P.Nx * P.dx, Ly = P.Ny * P.dy, Lz = P.Nz * P.dz;
    double R;
    if (P.ic_phi_seed_radius > 0.0) {
        R = P.ic_phi_seed_radius;
    } else {
        const double vf = std::fmin(0.999, std::fmax(1e-6, P.ic_vf_init_phi));
        R = std::fmax(1.0, is3d ? std::cbrt(vf * Lx * Ly * Lz / (n * (4.0 * PFGB_PI / 3.0)))
                                : std::sqrt(vf * Lx * Lz / (n * PFGB_PI)));
    }
    SeedGeom g;
    g.Nx = P.Nx; g.Ny = P.Ny; g.Nz = P.Nz; g.nseeds = n; g.is3d = is3d ? 1 : 0;
    g.dx = P.dx; g.dy = P.dy; g.dz = P.dz; g.Lx = Lx; g.Ly = Ly; g.Lz = Lz;
    g.w = P.ic_phi_iface_w > 0.0 ? P.ic_phi_iface_w * P.dx : P.dx;
    seed_axes(P, R, is3d, &g.Rx, &g.Ry, &g.Rz);
    g.min_axis = g.Rx;
    if (is3d && g.Ry < g.min_axis) g.min_axis = g.Ry;
    if (g.Rz < g.min_axis) g.min_axis = g.Rz;
    g.rotate = P.init_use_rotation && (P.init_tilt_theta_deg != 0.0 || P.init_tilt_phi_deg != 0.0);
    std::vector<double> tab = seed_centres(P);   // centres, then the rotations
    if (g.rotate) {
        double Rm[9];
        tilt_frame(P.init_tilt_theta_deg, P.init_tilt_phi_deg, Rm);
        for (int s = 0; s < n; ++s) tab.insert(tab.end(), Rm, Rm + 9);
    }
    double *d_tab = nullptr;
    INIT_TRY(cudaMalloc(&d_tab, sizeof(double) * tab.size()));
    cudaError_t e = cudaMemcpyAsync(d_tab, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, stream);
    const long long N = (long long)P.Nx * P.Ny * P.Nz;
    const unsigned long long nseed = P.init_phi_noise_seed != 0 ? P.init_phi_noise_seed : P.seed;
    if (e == cudaSuccess) {
        k_seed_phi<<<1216, 256, 0, stream>>>(g, d_tab, d_tab + 3 * n, d_phi, P.init_phi_noise_amp, nseed);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_h_moments<<<304, 256, 0, stream>>>(d_phi, N, d_scratch);
        e = cudaGetLastError();
    }
    std::vector<double> part(2 * 304);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(part.data(), d_scratch, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    cudaFree(d_tab);
    if (e != cudaSuccess) {
        pfgb_set_error_msg("seeded fields: %s", cudaGetErrorString(e));
        return PFGB_ERR_CUDA;
    }
    double sh = 0.0, sh2 = 0.0;
    for (int b = 0; b < 304; ++b) { sh += part[2 * b]; sh2 += part[2 * b + 1]; }
    const double mh = sh / (double)N, mh2 = sh2 / (double)N;
    const double xeq = P.xB_eq_matrix, vB = P.v_B;
    double xout;
    if (P.ic_23d_xB_out > 0.0) {
        xout = P.ic_23d_xB_out;
    } else {
        // <xB_tot> = A xB_out + B xB_eq + C with A = <(1-h)^2>, B = <h(1-h)>, C = v_B <h>
        const double vft = vf_target(P);
        const double target = vB * vft + (1.0 - vft) * xeq;
        const double A = 1.0 - 2.0 * mh + mh2, B = mh - mh2, C = vB * mh;
        if (std::fabs(A) < 1e-12) {
            const double den = std::fmax(1.0 - mh, 1e-12);
            xout = ((vft - mh) * vB + (1.0 - vft) * xeq) / den;
        } else {
            xout = (target - B * xeq - C) / A;
        }
    }
    xout = std::fmin(std::fmax(xout, P.xB_eps), 1.0 - P.xB_eps);
    k_seed_xB<<<1216, 256, 0, stream>>>(d_phi, d_xB, N, xout, xeq, P.xB_eps);
    INIT_TRY(cudaGetLastError());
    return PFGB_OK;
}

extern "C" pfgb_status pfgb_seed_fields(const pfgb_params *p, int device, double *phi, double *xB) {
    if (!p || !phi || !xB) return PFGB_ERR_INVALID;
    INIT_TRY(cudaSetDevice(device));
    const size_t N = (size_t)p->Nx * p->Ny * p->Nz;
    double *buf = nullptr;
    INIT_TRY(cudaMalloc(&buf, sizeof(double) * (2 * N + 2 * 304)));
    pfgb_status s = pfgb_seed_fields_device(p, buf, buf + N, buf + 2 * N, 0);
    cudaError_t e = cudaSuccess;
    if (s == PFGB_OK) e = cudaMemcpy(phi, buf, sizeof(double) * N, cudaMemcpyDeviceToHost);
    if (s == PFGB_OK && e == cudaSuccess) e = cudaMemcpy(xB, buf + N, sizeof(double) * N, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (s != PFGB_OK) return s;
    INIT_TRY(e);
    return PFGB_OK;
}

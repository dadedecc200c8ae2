// batch.cpp — batched minimize sweep over the C ABI: a queue of cases, a few
// host worker threads, one context (and CUDA stream) per running case so the
// small grids of a sweep share the device.
#include <atomic>
#include <cstdio>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "pfgb.h"

namespace {

pfgb_status run_case(pfgb_case *cs, int device) {
    const auto t0 = std::chrono::steady_clock::now();
    pfgb_ctx *ctx = nullptr;
    pfgb_status st = pfgb_create(&cs->params, device, &ctx);
    if (st != PFGB_OK) return st;
    cudaStream_t stream = nullptr;
    if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) {
        pfgb_destroy(ctx);
        return PFGB_ERR_CUDA;
    }
    st = pfgb_set_stream(ctx, stream);
    if (st == PFGB_OK) st = pfgb_load_fields(ctx, cs->phi, cs->xB, cs->eta, nullptr);
    const int n = cs->max_iter > 0 ? cs->max_iter : cs->params.minimize_max_iter;
    if (st == PFGB_OK) st = pfgb_minimize(ctx, n, cs->stop_on_convergence, &cs->stats);
    if (st == PFGB_OK && (cs->phi_out || cs->xB_out))
        st = pfgb_read_fields(ctx, cs->phi_out, cs->xB_out, nullptr, nullptr, nullptr);
    if (st == PFGB_OK) st = pfgb_sync(ctx);
    pfgb_destroy(ctx);
    cudaStreamDestroy(stream);
    cs->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return st;
}

// with fft_autotune, one iteration of the first case of each distinct grid
// on this thread before the worker threads start: the tiles are then timed on an
// otherwise idle device, and the cases find them chosen
void pretune(pfgb_case *cases, int ncases, int device) {
    std::vector<int> seen;
    for (int i = 0; i < ncases; ++i) {
        const pfgb_params &p = cases[i].params;
        if (!p.fft_autotune) continue;
        const int key[5] = {p.Nx, p.Ny, p.Nz, p.precision, p.model_mode};
        bool dup = false;
        for (size_t j = 0; j + 5 <= seen.size() && !dup; j += 5)
            dup = !memcmp(&seen[j], key, sizeof(key));
        if (dup) continue;
        seen.insert(seen.end(), key, key + 5);
        pfgb_ctx *ctx = nullptr;
        if (pfgb_create(&p, device, &ctx) != PFGB_OK) continue;
        if (pfgb_load_fields(ctx, cases[i].phi, cases[i].xB, cases[i].eta, nullptr) == PFGB_OK) {
            pfgb_min_stats st;
            pfgb_minimize(ctx, 1, 0, &st);
            pfgb_sync(ctx);
        }
        pfgb_destroy(ctx);
    }
}

}  // namespace

extern "C" pfgb_status pfgb_batch_minimize(pfgb_case *cases, int ncases, int device, int concurrency) {
    if (!cases || ncases < 0 || concurrency < 1) return PFGB_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return PFGB_ERR_CUDA;
    const int nt0 = concurrency < ncases ? concurrency : (ncases > 0 ? ncases : 1);
    pfgb_set_tune_copies(nt0);   // the tiles are chosen for nt0 cases sharing the device
    pretune(cases, ncases, device);
    pfgb_set_tune_copies(1);
    std::atomic<int> next(0);
    auto worker = [&]() {
        if (cudaSetDevice(device) != cudaSuccess) return;
        for (;;) {
            const int i = next.fetch_add(1);
            if (i >= ncases) return;
            cases[i].message[0] = '\0';
            cases[i].status = run_case(&cases[i], device);
            if (cases[i].status != PFGB_OK)
                snprintf(cases[i].message, sizeof(cases[i].message), "%s", pfgb_last_error(nullptr));
        }
    };
    for (int i = 0; i < ncases; ++i) cases[i].status = -1;
    std::vector<std::thread> pool;
    const int nt = concurrency < ncases ? concurrency : (ncases > 0 ? ncases : 1);
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto &th : pool) th.join();
    for (int i = 0; i < ncases; ++i)
        if (cases[i].status != PFGB_OK) return cases[i].status < 0 ? PFGB_ERR_CUDA : (pfgb_status)cases[i].status;
    return PFGB_OK;
}

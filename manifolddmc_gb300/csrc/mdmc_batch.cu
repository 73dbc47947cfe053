// mdmc_run_batch: many grids of uneven size per call.  A single grid of the
// batched workload (24..192 samples per axis) leaves most of the GPU idle and
// spends its time in launch gaps and the run's read-backs, so the batch runs
// the grids' pipelines concurrently: one context per grid slot (its buffers,
// and the mesh it returns) and S worker threads, each with its own stream,
// taking grids in turn.  S is chosen by timing the first batch with
// S = 1, 2, 4, 8, 16, 32 when the batch is created with streams = 0; the
// largest grids are started first.
// No counterpart in the reference (DualMarchingCubes::run takes one grid).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "mdmc.h"

struct mdmc_batch {
    mdmc_options opt;
    int streams = 0;  // 0: not chosen yet
    std::vector<mdmc_context*> ctx;
    std::vector<cudaStream_t> stream;
    std::string err;
};

namespace {

mdmc_status batchFail(mdmc_batch* b, mdmc_status st, const std::string& why) {
    if (b) b->err = why;
    return st;
}

mdmc_status ensureSlots(mdmc_batch* b, int n) {
    while ((int)b->ctx.size() < n) {
        mdmc_context* c = nullptr;
        const mdmc_status st = mdmc_create(&c, &b->opt);
        if (st != MDMC_OK) return batchFail(b, st, "mdmc_create failed for a batch slot");
        b->ctx.push_back(c);
    }
    return MDMC_OK;
}

mdmc_status ensureStreams(mdmc_batch* b, int s) {
    while ((int)b->stream.size() < s) {
        cudaStream_t st = nullptr;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
            return batchFail(b, MDMC_ERROR_CUDA, "cudaStreamCreate failed");
        b->stream.push_back(st);
    }
    return MDMC_OK;
}

// runs grids [0, n) on S workers; returns the first failing status
mdmc_status runWith(mdmc_batch* b, int S, const mdmc_grid* grids, const float* isos, int n, mdmc_mesh* meshes,
                    mdmc_stats* stats) {
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return batchFail(b, MDMC_ERROR_NO_DEVICE, "no current device");
    // largest grids first (cells as the work estimate), so that no large
    // grid starts last and runs alone
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto cells = [&](int i) {
        const int32_t* d = grids[i].dims;
        return (d[0] > 1 && d[1] > 1 && d[2] > 1) ? (int64_t)(d[0] - 1) * (d[1] - 1) * (d[2] - 1) : (int64_t)0;
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cells(a) > cells(c); });
    std::atomic<int> next{0};
    std::vector<mdmc_status> result(n, MDMC_OK);
    auto worker = [&](int w) {
        cudaSetDevice(device);
        for (int k = next.fetch_add(1); k < n; k = next.fetch_add(1)) {
            const int i = order[k];
            result[i] = mdmc_run(b->ctx[i], &grids[i], isos[i], meshes ? &meshes[i] : nullptr,
                                 stats ? &stats[i] : nullptr, b->stream[w]);
        }
    };
    if (S <= 1) {
        worker(0);
    } else {
        std::vector<std::thread> th;
        for (int w = 0; w < S; ++w) th.emplace_back(worker, w);
        for (auto& t : th) t.join();
    }
    for (int i = 0; i < n; ++i)
        if (result[i] != MDMC_OK && result[i] != MDMC_ERROR_LIMIT)
            return batchFail(b, result[i], "grid " + std::to_string(i) + ": " + mdmc_last_error(b->ctx[i]));
    return MDMC_OK;
}

}  // namespace

extern "C" {

mdmc_status mdmc_batch_create(mdmc_batch** batch, const mdmc_options* options, int streams) {
    if (!batch || streams < 0 || streams > 64) return MDMC_ERROR_INVALID_ARGUMENT;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        (void)cudaGetLastError();
        return MDMC_ERROR_NO_DEVICE;
    }
    mdmc_batch* b = new mdmc_batch();
    if (options) b->opt = *options;
    else mdmc_default_options(&b->opt);
    b->streams = streams;
    *batch = b;
    return MDMC_OK;
}

void mdmc_batch_destroy(mdmc_batch* b) {
    if (!b) return;
    for (mdmc_context* c : b->ctx) mdmc_destroy(c);
    for (cudaStream_t s : b->stream) cudaStreamDestroy(s);
    delete b;
}

mdmc_status mdmc_run_batch(mdmc_batch* b, const mdmc_grid* grids, const float* isos, int n, mdmc_mesh* meshes,
                           mdmc_stats* stats, void* stream) {
    if (!b || (n > 0 && (!grids || !isos)) || n < 0) return batchFail(b, MDMC_ERROR_INVALID_ARGUMENT, "bad arguments");
    b->err.clear();
    if (n == 0) return MDMC_OK;
    mdmc_status st = ensureSlots(b, n);
    if (st != MDMC_OK) return st;
    // the grids' inputs may still be in flight on the caller's stream
    if (stream) {
        if (cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
            return batchFail(b, MDMC_ERROR_CUDA, "caller stream failed");
    } else if (cudaDeviceSynchronize() != cudaSuccess) {
        return batchFail(b, MDMC_ERROR_CUDA, "device synchronize failed");
    }
    if (b->streams == 0) {
        // pick the worker count by timing this batch once per candidate
        const int candidates[] = {1, 2, 4, 8, 16, 32};
        double best = 1e30;
        int bestS = 1;
        if ((st = ensureStreams(b, 32)) != MDMC_OK) return st;
        for (int S : candidates) {
            if (S > std::max(n, 1)) break;
            const auto t0 = std::chrono::steady_clock::now();
            if ((st = runWith(b, S, grids, isos, n, meshes, stats)) != MDMC_OK) return st;
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (dt < best) {
                best = dt;
                bestS = S;
            }
        }
        b->streams = bestS;
    }
    if ((st = ensureStreams(b, b->streams)) != MDMC_OK) return st;
    return runWith(b, b->streams, grids, isos, n, meshes, stats);
}

int mdmc_batch_streams(const mdmc_batch* b) { return b ? b->streams : 0; }

mdmc_context* mdmc_batch_context(mdmc_batch* b, int i) {
    if (!b || i < 0 || i >= (int)b->ctx.size()) return nullptr;
    return b->ctx[i];
}

const char* mdmc_batch_last_error(const mdmc_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"

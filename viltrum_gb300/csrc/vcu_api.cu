/*
 * vcu_api.cu -- the extern "C" entry points of libviltrum_cuda.so (declared in
 * include/viltrum_cuda.h): context lifetime, argument validation, host<->device staging of the
 * caller's buffers, timing and device status.  The kernels live in k_*.cu.
 */
#include <cmath>
#include <new>

#include "vcu_internal.cuh"

namespace vcu {

int CallScope::begin() {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    VCU_CUDA(ctx, cudaSetDevice(ctx->device));
    VCU_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    VCU_CUDA(ctx, cudaEventRecord(ctx->ev_start, ctx->stream));
    return VCU_OK;
}

int CallScope::end(uint64_t evaluations, uint64_t regions) {
    VCU_CUDA(ctx, cudaEventRecord(ctx->ev_stop, ctx->stream));
    uint32_t flags = 0;
    VCU_CUDA(ctx, cudaMemcpyAsync(&flags, ctx->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    VCU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0.0f;
    VCU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    if (stats) {
        stats->device_ms = ms;
        stats->evaluations = evaluations;
        stats->regions = regions;
        stats->kernel_launches = launches;
        stats->flags = flags;
    }
    if (flags & VCU_FLAG_TIMEOUT) return fail(ctx, VCU_DEVICE_TIMEOUT, "a device-side wait expired");
    if (flags & VCU_FLAG_OVERFLOW) return fail(ctx, VCU_QUEUE_OVERFLOW, "a device queue overflowed");
    return VCU_OK;
}

/* output buffer: the caller's device pointer, or the context's staging buffer */
static int out_buffer(vcu_ctx* ctx, const vcu_problem* p, float* user, size_t bytes, float** dev) {
    if (p->mem == VCU_MEM_DEVICE) {
        *dev = user;
        return VCU_OK;
    }
    int rc = ensure(ctx, ctx->out, bytes);
    if (rc) return rc;
    *dev = static_cast<float*>(ctx->out.ptr);
    return VCU_OK;
}

int batch_launch(vcu_ctx* ctx, uint32_t& launches) {
    vcu_batch_state& B = ctx->batch;
    if (B.exec) {
        VCU_CUDA(ctx, cudaGraphLaunch(B.exec, ctx->stream));
    } else {
        /* the legacy default stream cannot be captured: launch directly */
        VCU_CUDA(ctx, cudaMemsetAsync(B.queue, 0, sizeof(uint32_t), ctx->stream));
        void* args[] = {&B.cfg, &B.items, &B.functors, &B.queue, &B.vals, &B.ranges,
                        &B.vols, &B.heap, &B.results, &B.item_ns, &ctx->d_status};
        VCU_CUDA(ctx, cudaLaunchKernel(B.kernel, dim3(B.blocks), dim3(B.threads), args, B.smem, ctx->stream));
    }
    ++launches;
    return VCU_OK;
}

int batch_capture(vcu_ctx* ctx, uint32_t& launches) {
    vcu_batch_state& B = ctx->batch;
    if (B.exec) {
        cudaGraphExecDestroy(B.exec);
        B.exec = nullptr;
    }
    B.valid = true;
    if (ctx->stream == nullptr) return batch_launch(ctx, launches);
    VCU_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    void* args[] = {&B.cfg, &B.items, &B.functors, &B.queue, &B.vals, &B.ranges,
                    &B.vols, &B.heap, &B.results, &B.item_ns, &ctx->d_status};
    cudaError_t e1 = cudaMemsetAsync(B.queue, 0, sizeof(uint32_t), ctx->stream);
    cudaError_t e2 = cudaLaunchKernel(B.kernel, dim3(B.blocks), dim3(B.threads), args, B.smem, ctx->stream);
    cudaGraph_t graph = nullptr;
    cudaError_t e3 = cudaStreamEndCapture(ctx->stream, &graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        B.valid = false;
        cudaGetLastError();
        return cuda_fail(ctx, e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3), "batch graph capture");
    }
    cudaError_t e4 = cudaGraphInstantiate(&B.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e4 != cudaSuccess) {
        B.exec = nullptr;
        B.valid = false;
        return cuda_fail(ctx, e4, "cudaGraphInstantiate");
    }
    return batch_launch(ctx, launches);
}

/* copy the batch results (and item times) out after a launch */
static int batch_finish(vcu_ctx* ctx, CallScope& scope, float* results, int32_t results_mem, vcu_batch_report* report) {
    vcu_batch_state& B = ctx->batch;
    const size_t bytes = B.n * sizeof(float);
    VCU_CUDA(ctx, cudaMemcpyAsync(results, B.results, bytes,
                                  results_mem == VCU_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                  ctx->stream));
    std::vector<uint64_t> ns;
    if (report && report->item_ms) {
        ns.resize(B.n);
        VCU_CUDA(ctx, cudaMemcpyAsync(ns.data(), B.item_ns, B.n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    const int rc = scope.end(B.evaluations, B.regions);
    if (report) {
        report->threads = B.threads;
        report->blocks = B.blocks;
        report->nested_regions = B.regions;
        if (report->item_ms)
            for (uint64_t i = 0; i < B.n; ++i) report->item_ms[i] = (float)((double)ns[i] * 1e-6);
    }
    return rc;
}

}  // namespace vcu

using namespace vcu;

extern "C" int vcu_integrate_batch(vcu_ctx* ctx, int32_t kind, const vcu_nested* nested, const vcu_batch_item* items,
                                   uint64_t n_items, float* results, int32_t results_mem, vcu_batch_report* report,
                                   vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    if (!items || !results || n_items == 0) return fail(ctx, VCU_INVALID_ARG, "empty batch or null results");
    if (n_items > 0x7fffffffull) return fail(ctx, VCU_INVALID_ARG, "too many batch items");
    if (results_mem != VCU_MEM_HOST && results_mem != VCU_MEM_DEVICE) return fail(ctx, VCU_INVALID_ARG, "bad results_mem");
    vcu_nested n{};
    if (nested) {
        n = *nested;
    } else {
        n.rule_hi = VCU_RULE_SIMPSON;
        n.rule_lo = VCU_RULE_TRAPEZOIDAL;
        n.heuristic = VCU_HEUR_DEFAULT;
        n.metric = VCU_METRIC_ABSOLUTE;
        n.size_weight = 1e-5;
        n.min_size = 1e-37;
        n.min_val = 1e-37;
    }
    CallScope scope{ctx, stats};
    int rc = scope.begin();
    if (rc) return rc;
    ctx->batch.valid = false;
    if (n.rule_hi == VCU_RULE_SIMPSON && n.rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_batch_st(ctx, kind, n, items, n_items, scope.launches);
    else if (n.rule_hi == VCU_RULE_BOOLE && n.rule_lo == VCU_RULE_SIMPSON)
        rc = run_batch_bs(ctx, kind, n, items, n_items, scope.launches);
    else if (n.rule_hi == VCU_RULE_BOOLE && n.rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_batch_bt(ctx, kind, n, items, n_items, scope.launches);
    else
        rc = fail(ctx, VCU_INVALID_ARG, "nested rules must be (simpson, trapezoidal), (boole, simpson) or (boole, trapezoidal)");
    if (rc) return rc;
    return batch_finish(ctx, scope, results, results_mem, report);
}

extern "C" int vcu_integrate_batch_resident(vcu_ctx* ctx, float* results, int32_t results_mem,
                                            vcu_batch_report* report, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    if (!ctx->batch.valid) return fail(ctx, VCU_INVALID_ARG, "no batch has been uploaded on this context");
    if (!results) return fail(ctx, VCU_INVALID_ARG, "null results");
    if (results_mem != VCU_MEM_HOST && results_mem != VCU_MEM_DEVICE) return fail(ctx, VCU_INVALID_ARG, "bad results_mem");
    CallScope scope{ctx, stats};
    int rc = scope.begin();
    if (rc) return rc;
    if ((rc = batch_launch(ctx, scope.launches))) return rc;
    return batch_finish(ctx, scope, results, results_mem, report);
}

extern "C" int vcu_abi_version(void) { return VCU_ABI_VERSION; }

extern "C" int vcu_create(vcu_ctx** out, const vcu_opts* opts) {
    if (!out) return VCU_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return VCU_NO_DEVICE;
    }
    vcu_ctx* ctx = new (std::nothrow) vcu_ctx();
    if (!ctx) return VCU_OOM;
    ctx->device = opts ? opts->device : 0;
    if (ctx->device < 0 || ctx->device >= ndev) {
        delete ctx;
        return VCU_INVALID_ARG;
    }
    auto bail = [&](cudaError_t e) {
        (void)e;
        cudaGetLastError();
        vcu_destroy(ctx);
        return VCU_CUDA_ERROR;
    };
    cudaError_t e;
    if ((e = cudaSetDevice(ctx->device)) != cudaSuccess) return bail(e);
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, ctx->device)) != cudaSuccess) return bail(e);
    ctx->sm_count = prop.multiProcessorCount;
    ctx->smem_optin = prop.sharedMemPerBlockOptin;
    if (opts && opts->stream) {
        ctx->stream = static_cast<cudaStream_t>(opts->stream);
        ctx->own_stream = false;
    } else {
        if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
        ctx->own_stream = true;
    }
    if ((e = cudaEventCreate(&ctx->ev_start)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&ctx->ev_stop)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&ctx->ev_tune[0])) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreate(&ctx->ev_tune[1])) != cudaSuccess) return bail(e);
    if ((e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking)) != cudaSuccess) return bail(e);
    if ((e = cudaEventCreateWithFlags(&ctx->ev_snap, cudaEventDisableTiming)) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc(&ctx->d_status, 256)) != cudaSuccess) return bail(e);
    if ((e = cudaMemset(ctx->d_status, 0, 256)) != cudaSuccess) return bail(e);
    *out = ctx;
    return VCU_OK;
}

extern "C" int vcu_destroy(vcu_ctx* ctx) {
    if (!ctx) return VCU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->batch.exec) cudaGraphExecDestroy(ctx->batch.exec);
    for (vcu_buffer* b : {&ctx->out, &ctx->aux, &ctx->in, &ctx->scratch, &ctx->batch_in, &ctx->batch_pool})
        if (b->ptr) cudaFree(b->ptr);
    if (ctx->d_status) cudaFree(ctx->d_status);
    if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
    if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
    for (cudaEvent_t ev : ctx->ev_tune)
        if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->ev_snap) cudaEventDestroy(ctx->ev_snap);
    cudaGetLastError();
    delete ctx;
    return VCU_OK;
}

extern "C" int vcu_set_device_memory_limit(vcu_ctx* ctx, uint64_t bytes) {
    if (!ctx) return VCU_INVALID_ARG;
    ctx->mem_limit = bytes;
    return VCU_OK;
}

extern "C" uint64_t vcu_device_memory_held(const vcu_ctx* ctx) { return ctx ? (uint64_t)ctx->held : 0; }

extern "C" int vcu_last_error(const vcu_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return VCU_INVALID_ARG;
    std::snprintf(buf, len, "%s", ctx->last_error.c_str());
    return VCU_OK;
}

extern "C" int vcu_channels(int32_t kind) {
    switch (kind) {
    case VCU_F_POLY2: case VCU_F_SIN1: case VCU_F_SPHERE3: case VCU_F_WAVE2: case VCU_F_SCENE2:
    case VCU_F_HALFSPACE: case VCU_F_OCCLUDED_SCENE5: case VCU_F_WALK2:
        return 1;
    case VCU_F_MOVING_SCENE3:
        return 3;
    default:
        return -VCU_INVALID_ARG;
    }
}

extern "C" int vcu_eval(vcu_ctx* ctx, const vcu_integrand* f, int32_t dim, const float* x, int64_t npts, float* out,
                        int32_t mem) {
    if (!ctx) return VCU_INVALID_ARG;
    if (!f || npts < 0 || (npts > 0 && (!x || !out))) return fail(ctx, VCU_INVALID_ARG, "bad vcu_eval arguments");
    const int ch = vcu_channels(f->kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, nullptr};
    int rc = scope.begin();
    if (rc) return rc;
    const float* dx = x;
    float* dout = out;
    if (mem == VCU_MEM_HOST && npts > 0) {
        if ((rc = ensure(ctx, ctx->in, (size_t)npts * dim * 4))) return rc;
        if ((rc = ensure(ctx, ctx->out, (size_t)npts * ch * 4))) return rc;
        VCU_CUDA(ctx, cudaMemcpyAsync(ctx->in.ptr, x, (size_t)npts * dim * 4, cudaMemcpyHostToDevice, ctx->stream));
        dx = static_cast<float*>(ctx->in.ptr);
        dout = static_cast<float*>(ctx->out.ptr);
    }
    if ((rc = run_eval(ctx, *f, dim, dx, npts, dout, scope.launches))) return rc;
    if (mem == VCU_MEM_HOST && npts > 0)
        VCU_CUDA(ctx, cudaMemcpyAsync(out, dout, (size_t)npts * ch * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return scope.end((uint64_t)npts, 0);
}

static int per_bin_mc(vcu_ctx* ctx, const vcu_problem* p, uint64_t spp, uint64_t seed, const float* points, float* bins,
                      bool accumulate, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (spp == 0 || spp > 0xffffffffull) return fail(ctx, VCU_INVALID_ARG, "samples per bin must be 1..2^32-1");
    if (!bins) return fail(ctx, VCU_INVALID_ARG, "null bins");
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    float* dbins = nullptr;
    if ((rc = out_buffer(ctx, p, bins, g.nbins * ch * 4, &dbins))) return rc;
    if (accumulate && p->mem == VCU_MEM_HOST)
        VCU_CUDA(ctx, cudaMemcpyAsync(dbins, bins, g.nbins * ch * 4, cudaMemcpyHostToDevice, ctx->stream));
    const float* dpts = points;
    if (points && p->mem == VCU_MEM_HOST) {
        const size_t bytes = g.nbins * spp * p->dim * 4;
        if ((rc = ensure(ctx, ctx->in, bytes))) return rc;
        VCU_CUDA(ctx, cudaMemcpyAsync(ctx->in.ptr, points, bytes, cudaMemcpyHostToDevice, ctx->stream));
        dpts = static_cast<const float*>(ctx->in.ptr);
    }
    if ((rc = run_mc(ctx, p, g, spp, seed, dpts, dbins, accumulate, scope.launches))) return rc;
    if (p->mem == VCU_MEM_HOST)
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, g.nbins * ch * 4, cudaMemcpyDeviceToHost, ctx->stream));
    return scope.end(g.nbins * spp, 0);
}

extern "C" int vcu_per_bin_monte_carlo(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin, uint64_t seed,
                                       float* bins, vcu_stats* stats) {
    return per_bin_mc(ctx, p, samples_per_bin, seed, nullptr, bins, false, stats);
}

extern "C" int vcu_per_bin_monte_carlo_replay(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin,
                                              const float* points, float* bins, vcu_stats* stats) {
    if (ctx && !points) return fail(ctx, VCU_INVALID_ARG, "null points");
    return per_bin_mc(ctx, p, samples_per_bin, 0, points, bins, false, stats);
}

extern "C" int vcu_per_bin_monte_carlo_accumulate(vcu_ctx* ctx, const vcu_problem* p, uint64_t samples_per_bin,
                                                  uint64_t seed, const float* points, float* bins, vcu_stats* stats) {
    return per_bin_mc(ctx, p, samples_per_bin, seed, points, bins, true, stats);
}

extern "C" int vcu_per_bin_adaptive_nested(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested,
                                           uint64_t iterations, float* bins, int32_t* trace, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (!nested || !bins) return fail(ctx, VCU_INVALID_ARG, "null nested rule or bins");
    if (iterations > 62) return fail(ctx, VCU_UNSUPPORTED, "per-bin region budget is limited to 62 splits (63 regions)");
    if ((rc = check_per_bin_nested(ctx, *nested))) return rc;
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    float* dbins = nullptr;
    if ((rc = out_buffer(ctx, p, bins, g.nbins * ch * 4, &dbins))) return rc;
    int32_t* dtrace = trace;
    const size_t tbytes = g.nbins * iterations * 2 * 4;
    if (trace && p->mem == VCU_MEM_HOST) {
        if ((rc = ensure(ctx, ctx->aux, tbytes))) return rc;
        dtrace = static_cast<int32_t*>(ctx->aux.ptr);
    }
    if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_SIMPSON)
        rc = run_nested_bs(ctx, p, g, *nested, (int)iterations, dbins, dtrace, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_nested_bt(ctx, p, g, *nested, (int)iterations, dbins, dtrace, scope.launches);
    else if (nested->rule_hi == VCU_RULE_SIMPSON && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_nested_st(ctx, p, g, *nested, (int)iterations, dbins, dtrace, scope.launches);
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST) {
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, g.nbins * ch * 4, cudaMemcpyDeviceToHost, ctx->stream));
        if (trace) VCU_CUDA(ctx, cudaMemcpyAsync(trace, dtrace, tbytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    /* evaluations: root S^dim + iterations x (S-1) S^(dim-1) per bin */
    const int S = nested->rule_hi;
    double sd = 1.0, sd1 = 1.0;
    for (int d = 0; d < p->dim; ++d) sd *= S;
    for (int d = 0; d < p->dim - 1; ++d) sd1 *= S;
    const uint64_t evals = (uint64_t)((double)g.nbins * (sd + (double)iterations * (S - 1) * sd1));
    return scope.end(evals, g.nbins * (iterations + 1));
}

extern "C" int vcu_cv_replay_width(int32_t dim, int32_t sampling) {
    return 1 + dim + (sampling == VCU_RS_RUSSIAN_ROULETTE ? 1 : sampling == VCU_RS_MIS ? 1 + dim : 0);
}

extern "C" int vcu_control_variates(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested, uint64_t iterations,
                                    const vcu_cv* cv, const float* replay, float* bins, float* approximation,
                                    float* regions, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (!nested || !cv || !bins) return fail(ctx, VCU_INVALID_ARG, "null nested rule, cv options or bins");
    if (iterations >= (1ull << 23)) return fail(ctx, VCU_UNSUPPORTED, "control variates take at most 2^23-1 splits");
    if (cv->samples_per_bin > 0xffffffffull) return fail(ctx, VCU_INVALID_ARG, "samples per bin must be < 2^32");
    if (cv->weight != VCU_CV_OPTIMIZE && cv->weight != VCU_CV_FIXED) return fail(ctx, VCU_INVALID_ARG, "unknown weight");
    if (cv->reserved != 0 || cv->reserved2 != 0) return fail(ctx, VCU_INVALID_ARG, "vcu_cv::reserved must be 0");
    if (cv->rr < VCU_RR_UNIFORM || cv->rr > VCU_RR_PDF) return fail(ctx, VCU_INVALID_ARG, "unknown residual region choice");
    if (cv->sampling < VCU_RS_UNIFORM || cv->sampling > VCU_RS_MIS)
        return fail(ctx, VCU_INVALID_ARG, "unknown residual point sampling");
    if ((cv->rr == VCU_RR_PDF || cv->sampling != VCU_RS_UNIFORM) && nested->rule_hi != VCU_RULE_SIMPSON)
        return fail(ctx, VCU_UNSUPPORTED, "the pdf strategies need a Simpson high rule (rules.h:102-248)");
    const bool fubini = cv->fubini_dims != 0;
    if (fubini) {
        const bool unbounded = p->f.kind == VCU_F_WALK2; /* its tail has no finite dimension */
        if (cv->fubini_dims != 2 || (p->dim < 3 && !unbounded) || p->dimbins > 2)
            return fail(ctx, VCU_UNSUPPORTED, "a Fubini tail takes regions over 2 dimensions of a 3+ dimensional "
                                              "integrand, at most 2 of them binned");
        if (cv->tail_samples == 0) return fail(ctx, VCU_INVALID_ARG, "tail_samples must be >= 1");
        if (nested->rule_hi != VCU_RULE_SIMPSON || nested->rule_lo != VCU_RULE_TRAPEZOIDAL)
            return fail(ctx, VCU_UNSUPPORTED, "a Fubini tail is built for nested(simpson, trapezoidal)");
    }
    const int rdim = fubini ? cv->fubini_dims : p->dim; /* dimensions of the regions */
    if (nested->heuristic != VCU_HEUR_DEFAULT && nested->heuristic != VCU_HEUR_SIZE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error heuristic");
    if (nested->metric != VCU_METRIC_ABSOLUTE && nested->metric != VCU_METRIC_RELATIVE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error metric");
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    const size_t bbytes = g.nbins * ch * 4, rbytes = (iterations + 1) * 2 * rdim * 4, vbytes = g.nbins * 4;
    float *dbins = bins, *dapprox = approximation, *dregions = regions;
    const float* dreplay = replay;
    vcu_cv cvd = *cv; /* with the variance output moved to device memory */
    if (p->mem == VCU_MEM_HOST) {
        const size_t bb = (bbytes + 255) & ~size_t(255), rb = (rbytes + 255) & ~size_t(255);
        if ((rc = ensure(ctx, ctx->out, 2 * bb + rb + vbytes + 512))) return rc;
        char* o = static_cast<char*>(ctx->out.ptr);
        dbins = reinterpret_cast<float*>(o);
        dapprox = approximation ? reinterpret_cast<float*>(o + bb) : nullptr;
        dregions = regions ? reinterpret_cast<float*>(o + 2 * bb) : nullptr;
        cvd.variance = cv->variance ? reinterpret_cast<float*>(o + 2 * bb + rb) : nullptr;
        if (replay) {
            const size_t pbytes = g.nbins * cv->samples_per_bin * (size_t)vcu_cv_replay_width(rdim, cv->sampling) * 4;
            if ((rc = ensure(ctx, ctx->in, pbytes))) return rc;
            VCU_CUDA(ctx, cudaMemcpyAsync(ctx->in.ptr, replay, pbytes, cudaMemcpyHostToDevice, ctx->stream));
            dreplay = static_cast<const float*>(ctx->in.ptr);
        }
    }
    const int it = (int)iterations;
    if (nested->rule_hi == VCU_RULE_SIMPSON && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = fubini ? run_cv_fubini(ctx, p, g, *nested, it, cvd, dreplay, dbins, dapprox, dregions, scope.launches)
                    : run_cv_st(ctx, p, g, *nested, it, cvd, dreplay, dbins, dapprox, dregions, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_SIMPSON)
        rc = run_cv_bs(ctx, p, g, *nested, it, cvd, dreplay, dbins, dapprox, dregions, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_cv_bt(ctx, p, g, *nested, it, cvd, dreplay, dbins, dapprox, dregions, scope.launches);
    else
        rc = fail(ctx, VCU_INVALID_ARG, "unsupported nested rule pair");
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST) {
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (approximation) VCU_CUDA(ctx, cudaMemcpyAsync(approximation, dapprox, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (regions) VCU_CUDA(ctx, cudaMemcpyAsync(regions, dregions, rbytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (cv->variance)
            VCU_CUDA(ctx, cudaMemcpyAsync(cv->variance, cvd.variance, vbytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    const int S = nested->rule_hi;
    double sd = 1.0, sd1 = 1.0;
    for (int d = 0; d < rdim; ++d) sd *= S;
    for (int d = 0; d < rdim - 1; ++d) sd1 *= S;
    const double per_node = fubini ? (double)cv->tail_samples : 1.0; /* integrand calls per node value */
    const uint64_t evals =
        (uint64_t)((sd + (double)iterations * (S - 1) * sd1) * per_node) + g.nbins * cv->samples_per_bin;
    return scope.end(evals, iterations + 1);
}

extern "C" int vcu_adaptive_iterations_global(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested,
                                              uint64_t iterations, float* bins, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (!nested || !bins) return fail(ctx, VCU_INVALID_ARG, "null nested rule or bins");
    if (iterations >= (1ull << 23)) return fail(ctx, VCU_UNSUPPORTED, "at most 2^23-1 splits");
    if (nested->heuristic != VCU_HEUR_DEFAULT && nested->heuristic != VCU_HEUR_SIZE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error heuristic");
    if (nested->metric != VCU_METRIC_ABSOLUTE && nested->metric != VCU_METRIC_RELATIVE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error metric");
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    const size_t bbytes = g.nbins * ch * 4;
    float* dbins = bins;
    if (p->mem == VCU_MEM_HOST) {
        if ((rc = ensure(ctx, ctx->out, bbytes + 256))) return rc;
        dbins = static_cast<float*>(ctx->out.ptr);
        VCU_CUDA(ctx, cudaMemcpyAsync(dbins, bins, bbytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    /* the control-variate pipeline without residual samples: its approximation, started from the
     * bins' current values, is exactly the sequential regions integrator's accumulation */
    vcu_cv cv{};
    cv.samples_per_bin = 0;
    cv.weight = VCU_CV_FIXED;
    cv.reserved = 1;
    cv.alpha = 1.0;
    const int it = (int)iterations;
    if (nested->rule_hi == VCU_RULE_SIMPSON && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_cv_st(ctx, p, g, *nested, it, cv, nullptr, dbins, nullptr, nullptr, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_SIMPSON)
        rc = run_cv_bs(ctx, p, g, *nested, it, cv, nullptr, dbins, nullptr, nullptr, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_cv_bt(ctx, p, g, *nested, it, cv, nullptr, dbins, nullptr, nullptr, scope.launches);
    else
        rc = fail(ctx, VCU_INVALID_ARG, "unsupported nested rule pair");
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST)
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
    const int S = nested->rule_hi;
    double sd = 1.0, sd1 = 1.0;
    for (int d = 0; d < p->dim; ++d) sd *= S;
    for (int d = 0; d < p->dim - 1; ++d) sd1 *= S;
    return scope.end((uint64_t)(sd + (double)iterations * (S - 1) * sd1), iterations + 1);
}

extern "C" int vcu_adaptive_tolerance(vcu_ctx* ctx, const vcu_problem* p, const vcu_nested* nested, float tolerance,
                                      uint64_t max_regions, float* bins, uint64_t* leaves, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (!nested || !bins) return fail(ctx, VCU_INVALID_ARG, "null nested rule or bins");
    if (!(tolerance > 0.0f)) return fail(ctx, VCU_INVALID_ARG, "tolerance must be positive");
    if (nested->heuristic != VCU_HEUR_DEFAULT && nested->heuristic != VCU_HEUR_SIZE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error heuristic");
    if (nested->metric != VCU_METRIC_ABSOLUTE && nested->metric != VCU_METRIC_RELATIVE)
        return fail(ctx, VCU_INVALID_ARG, "unknown error metric");
    const int ch = vcu_channels(p->f.kind);
    if (ch < 0) return fail(ctx, VCU_INVALID_ARG, "unknown integrand kind");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    const size_t bbytes = g.nbins * ch * 4;
    float* dbins = bins;
    if (p->mem == VCU_MEM_HOST) {
        if ((rc = ensure(ctx, ctx->out, bbytes + 256))) return rc;
        dbins = static_cast<float*>(ctx->out.ptr);
        VCU_CUDA(ctx, cudaMemcpyAsync(dbins, bins, bbytes, cudaMemcpyHostToDevice, ctx->stream));
    }
    uint64_t nregions = 0, nleaves = 0;
    if (nested->rule_hi == VCU_RULE_SIMPSON && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_tol_st(ctx, p, g, *nested, tolerance, max_regions, dbins, nregions, nleaves, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_SIMPSON)
        rc = run_tol_bs(ctx, p, g, *nested, tolerance, max_regions, dbins, nregions, nleaves, scope.launches);
    else if (nested->rule_hi == VCU_RULE_BOOLE && nested->rule_lo == VCU_RULE_TRAPEZOIDAL)
        rc = run_tol_bt(ctx, p, g, *nested, tolerance, max_regions, dbins, nregions, nleaves, scope.launches);
    else
        rc = fail(ctx, VCU_INVALID_ARG, "unsupported nested rule pair");
    if (rc) return rc;
    if (p->mem == VCU_MEM_HOST)
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
    if (leaves) *leaves = nleaves;
    const int S = nested->rule_hi;
    double sd = 1.0, sd1 = 1.0;
    for (int d = 0; d < p->dim; ++d) sd *= S;
    for (int d = 0; d < p->dim - 1; ++d) sd1 *= S;
    const uint64_t splits = nregions > 0 ? (nregions - 1) / 2 : 0;
    return scope.end((uint64_t)(sd + (double)splits * (S - 1) * sd1), nregions);
}

extern "C" int vcu_learned_control_variates(vcu_ctx* ctx, const vcu_problem* p, const vcu_learned* opt, float* bins,
                                            float* network_integral, vcu_learned_report* report, vcu_stats* stats) {
    if (!ctx) return VCU_INVALID_ARG;
    BinGrid g;
    int rc = make_grid(ctx, p, g);
    if (rc) return rc;
    if (!opt || !bins) return fail(ctx, VCU_INVALID_ARG, "null options or bins");
    if (opt->cells < 0 || opt->cells > 64 || opt->cells_unbinned < 1 || opt->cells_unbinned > 64)
        return fail(ctx, VCU_INVALID_ARG, "cells must be 0..64 and cells_unbinned 1..64");
    {
        double nodes = 1.0;
        for (int d = 0; d < p->dim; ++d) nodes *= d < p->dimbins ? 2 * opt->cells + 1 : 2 * opt->cells_unbinned + 1;
        if (nodes > 4913.0) return fail(ctx, VCU_UNSUPPORTED, "at most 4913 interpolation nodes per bin");
    }
    if (opt->samples_per_bin == 0 || opt->samples_per_bin > 0xffffffffull)
        return fail(ctx, VCU_INVALID_ARG, "samples per bin must be 1..2^32-1");
    if (opt->train_steps > 0 && opt->batch == 0) return fail(ctx, VCU_INVALID_ARG, "batch must be positive");
    if ((opt->poly_bins == nullptr) != (opt->poly_variance == nullptr))
        return fail(ctx, VCU_INVALID_ARG, "poly_bins and poly_variance go together");
    if (vcu_channels(p->f.kind) != 1) return fail(ctx, VCU_UNSUPPORTED, "learned control variates take scalar integrands");
    CallScope scope{ctx, stats};
    if ((rc = scope.begin())) return rc;
    float *dbins = bins, *dint = network_integral;
    vcu_learned o = *opt; /* with the polynomial estimates moved to device memory */
    const size_t bbytes = g.nbins * 4, bb = (bbytes + 255) & ~size_t(255);
    if (p->mem == VCU_MEM_HOST) {
        if ((rc = ensure(ctx, ctx->out, 4 * bb + 512))) return rc;
        char* base = static_cast<char*>(ctx->out.ptr);
        dbins = reinterpret_cast<float*>(base);
        dint = network_integral ? reinterpret_cast<float*>(base + bb) : nullptr;
        if (opt->poly_bins) {
            float* pb = reinterpret_cast<float*>(base + 2 * bb);
            float* pv = reinterpret_cast<float*>(base + 3 * bb);
            VCU_CUDA(ctx, cudaMemcpyAsync(pb, opt->poly_bins, bbytes, cudaMemcpyHostToDevice, ctx->stream));
            VCU_CUDA(ctx, cudaMemcpyAsync(pv, opt->poly_variance, bbytes, cudaMemcpyHostToDevice, ctx->stream));
            o.poly_bins = pb;
            o.poly_variance = pv;
        }
    }
    vcu_learned_report rep{};
    if ((rc = run_learned(ctx, p, g, o, dbins, dint, &rep, scope.launches))) return rc;
    if (report) *report = rep;
    if (p->mem == VCU_MEM_HOST) {
        VCU_CUDA(ctx, cudaMemcpyAsync(bins, dbins, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
        if (network_integral)
            VCU_CUDA(ctx, cudaMemcpyAsync(network_integral, dint, bbytes, cudaMemcpyDeviceToHost, ctx->stream));
    }
    /* integrand evaluations: training and held-out samples, then pilot + residual samples per bin */
    const uint64_t pilot = opt->fallback ? learned_pilot(opt->samples_per_bin, opt->pilot) : 0;
    const uint64_t evals = (uint64_t)rep.train_steps_run * opt->batch + g.nbins * (opt->samples_per_bin + pilot);
    return scope.end(evals, 0);
}

extern "C" int vcu_mlp_eval(vcu_ctx* ctx, int32_t dim, const float* theta, const float* u, const float* y,
                            int64_t npts, float* out, float* grad) {
    if (!ctx) return VCU_INVALID_ARG;
    if (!theta || !u || !out || npts <= 0) return fail(ctx, VCU_INVALID_ARG, "bad vcu_mlp_eval arguments");
    if (grad && !y) return fail(ctx, VCU_INVALID_ARG, "the gradient needs targets y");
    CallScope scope{ctx, nullptr};
    int rc = scope.begin();
    if (rc) return rc;
    if ((rc = run_mlp_eval(ctx, dim, theta, u, y, npts, out, grad, scope.launches))) return rc;
    return scope.end((uint64_t)npts, 0);
}

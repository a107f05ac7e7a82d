// Reducer plumbing shared by k_reduce.cu and k_canon.cu.
#pragma once

#include <cstring>

#include "kcommon.cuh"
#include "registry.h"

namespace vkc {

// A reducer whose running state is a small device buffer owned by the reducer.
struct DevReducer : ReducerImpl {
    void *state = nullptr;
    size_t bytes = 0;
    DeviceMem mem;  // frees `state` on the context's stream, even after the context closed
    // Allocates the zeroed state.
    vkc_status alloc(vkc_ctx *ctx, size_t n) {
        bytes = n;
        VKC_CUDA(ctx, cudaMallocAsync(&state, n, ctx->stream));
        mem.ptr = state;
        mem.box = ctx->box;
        VKC_CUDA(ctx, cudaMemsetAsync(state, 0, n, ctx->stream));
        return VKC_OK;
    }
    vkc_status upload(vkc_ctx *ctx, const void *h, size_t n, size_t at = 0) {
        void *p;
        vkc_status st = pinned(ctx, n, &p);
        if (st) return st;
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        memcpy(p, h, n);
        VKC_CUDA(ctx, cudaMemcpyAsync(static_cast<char *>(state) + at, p, n,
                                      cudaMemcpyHostToDevice, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return VKC_OK;
    }
    vkc_status download(vkc_ctx *ctx, void *h, size_t n, size_t at = 0) {
        void *p;
        vkc_status st = pinned(ctx, n, &p);
        if (st) return st;
        VKC_CUDA(ctx, cudaMemcpyAsync(p, static_cast<char *>(state) + at, n,
                                      cudaMemcpyDeviceToHost, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        memcpy(h, p, n);
        return VKC_OK;
    }
};

CmpRange cmp_range(int cmp, double c);
void register_canon(std::vector<KernelDef> &t);

}  // namespace vkc

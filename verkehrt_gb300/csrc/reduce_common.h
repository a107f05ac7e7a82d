// Reducer plumbing shared by k_reduce.cu and k_canon.cu.
#pragma once

#include <cstring>

#include "kcommon.cuh"
#include "registry.h"

namespace vkc {

// Up to four 8-byte words that a fill repeats over a reducer's state.
struct Words4 {
    unsigned long long w[4];
};

// Word i of the state gets w.w[i < 4 ? i : 3].
static __global__ void reducer_fill_kernel(unsigned long long *p, int n, Words4 w) {
    const int i = threadIdx.x;
    if (i < n) p[i] = w.w[i < 4 ? i : 3];
}

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
    // The state's first n words set on the device (a launch, so it can be captured): word i
    // gets w_i for i < 3, the rest w3.
    vkc_status fill(vkc_ctx *ctx, int n, unsigned long long w0, unsigned long long w1 = 0,
                    unsigned long long w2 = 0, unsigned long long w3 = 0) {
        reducer_fill_kernel<<<1, 64, 0, ctx->stream>>>(static_cast<unsigned long long *>(state), n,
                                                       Words4{{w0, w1, w2, w3}});
        return launched(ctx, "reducer_fill");
    }
    // n bytes of the state from byte `at` to the device address dst, on the context's stream.
    vkc_status copy_out(vkc_ctx *ctx, void *dst, size_t n, size_t at = 0) {
        VKC_CUDA(ctx, cudaMemcpyAsync(dst, static_cast<const char *>(state) + at, n,
                                      cudaMemcpyDeviceToDevice, ctx->stream));
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

// capi.cu - context lifetime, error reporting and host/device staging.
#include "common.cuh"

mptg_status mptg_fail(mptg_ctx* ctx, mptg_status st, const char* fmt, ...) {
    if (ctx) {
        char msg[sizeof(ctx->err)];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(msg, sizeof(msg), fmt, ap);
        va_end(ap);
        // batch workers may fail concurrently on one context
        std::lock_guard<std::mutex> lock(ctx->mu);
        memcpy(ctx->err, msg, sizeof(msg));
    }
    return st;
}

bool mptg_is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

mptg_status mptg_stage_in(mptg_ctx* ctx, const void* user, size_t bytes, cudaStream_t s, DevBuf* out) {
    out->user = user;
    out->bytes = bytes;
    if (bytes == 0) { out->dptr = nullptr; out->owned = false; return MPTG_OK; }
    if (mptg_is_device_ptr(user)) {
        out->dptr = const_cast<void*>(user);
        out->owned = false;
        return MPTG_OK;
    }
    MPTG_CUDA_TRY(ctx, cudaMallocAsync(&out->dptr, bytes, s));
    out->owned = true;
    MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(out->dptr, user, bytes, cudaMemcpyHostToDevice, s));
    return MPTG_OK;
}

mptg_status mptg_stage_out_alloc(mptg_ctx* ctx, void* user, size_t bytes, cudaStream_t s, DevBuf* out) {
    out->user = user;
    out->bytes = bytes;
    if (bytes == 0 || user == nullptr) { out->dptr = nullptr; out->owned = false; return MPTG_OK; }
    if (mptg_is_device_ptr(user)) {
        out->dptr = user;
        out->owned = false;
        return MPTG_OK;
    }
    MPTG_CUDA_TRY(ctx, cudaMallocAsync(&out->dptr, bytes, s));
    out->owned = true;
    return MPTG_OK;
}

mptg_status mptg_stage_finish(mptg_ctx* ctx, cudaStream_t s, DevBuf* outs, int nouts, DevBuf* ins, int nins) {
    bool sync = false;
    for (int i = 0; i < nouts; ++i) {
        if (outs[i].owned) {
            MPTG_CUDA_TRY(ctx, cudaMemcpyAsync(const_cast<void*>(outs[i].user), outs[i].dptr, outs[i].bytes,
                                               cudaMemcpyDeviceToHost, s));
            MPTG_CUDA_TRY(ctx, cudaFreeAsync(outs[i].dptr, s));
            sync = true;
        }
    }
    for (int i = 0; i < nins; ++i) {
        if (ins[i].owned) {
            MPTG_CUDA_TRY(ctx, cudaFreeAsync(ins[i].dptr, s));
            sync = true;
        }
    }
    if (sync) MPTG_CUDA_TRY(ctx, cudaStreamSynchronize(s));
    return MPTG_OK;
}

extern "C" {

mptg_status mptg_create(mptg_ctx** out, int device) {
    if (!out) return MPTG_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return MPTG_ERR_CUDA;
    }
    if (device < 0 || device >= n) return MPTG_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return MPTG_ERR_CUDA;
    mptg_ctx* c = new mptg_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    *out = c;
    return MPTG_OK;
}

mptg_status mptg_destroy(mptg_ctx* ctx) {
    if (!ctx) return MPTG_ERR_INVALID_ARG;
    delete ctx;
    return MPTG_OK;
}

const char* mptg_last_error(mptg_ctx* ctx) {
    return ctx ? ctx->err : "null context";
}

uint64_t mptg_kernel_launches(mptg_ctx* ctx) {
    return ctx ? ctx->launches.load() : 0;
}

}  // extern "C"

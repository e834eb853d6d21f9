// The C ABI of include/halcuda.h, part 1: contexts, device tensors and the Backend methods.
// Host-side argument checks mirror the assertions of the reference implementation
// (cyclosubfield-dbfv/src/hal/cpu.rs) and turn them into status codes.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

struct hc_context_s {
    int device;
    cudaStream_t own;
    cudaStream_t stream;
    uint64_t launches;
    int sms;
    size_t smem_optin;
};

struct hc_perm_plan_s {
    uint32_t* dev;
    size_t len;
};

namespace hc {

thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }
hc_status fail(hc_status st, const std::string& msg) {
    g_error = msg;
    return st;
}
hc_status cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return HC_OK;
    return fail(e == cudaErrorMemoryAllocation ? HC_ERR_OOM : HC_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
cudaStream_t stream_of(hc_context ctx) { return ctx->stream; }
static std::atomic<uint64_t> g_alloc_calls{0};
void count_alloc() { g_alloc_calls.fetch_add(1, std::memory_order_relaxed); }
uint64_t alloc_calls() { return g_alloc_calls.load(std::memory_order_relaxed); }
void count_launch(hc_context ctx, uint64_t n) { ctx->launches += n; }
uint64_t launch_counter(hc_context ctx) { return ctx->launches; }
int num_sms(hc_context ctx) { return ctx->sms; }
size_t max_smem_optin(hc_context ctx) { return ctx->smem_optin; }
int device_of(hc_context ctx) { return ctx->device; }

// defined in ntt.cu / ops.cu
hc_status build_plan(hc_context ctx, const hc_modulus* m, const size_t* shape, size_t k, hc_ntt_plan* out);
hc_status destroy_plan(hc_ntt_plan p);
hc_status launch_ntt(hc_context ctx, const KView& t, const hc_ntt_plan* plans, size_t nplans, int dim, int mode,
                     const KView& mul, const KMods& mods, const KView* src = nullptr);
bool ntt_column_path(const hc_ntt_plan* plans, size_t nplans, int dim);
hc_status launch_pointwise(hc_context ctx, int op, const KView& d, const KView& a, const KView& b, const KMods& m);
hc_status launch_matmul(hc_context ctx, const KView& d, const KView& lhs, const KView& rhs, int64_t U);
hc_status launch_inner_product(hc_context ctx, const KView& d, const KView* l, const KView* r, int n);
hc_status launch_bconv_correct(hc_context ctx, const KView& d, const KView& lhs, const KView& rhs, const KMods& m,
                               int shift);
hc_status launch_bconv_pow2(hc_context ctx, const KView& d, const KView& src, i128 f0, i128 f1, int shift, int log2m,
                            int wide);
hc_status launch_permute(hc_context ctx, const KView& d, const KView& s, const uint32_t* perm, int dim);

}  // namespace hc

using namespace hc;

namespace {

enum PwOp {  // keep in sync with ops.cu
    OP_ASSIGN,
    OP_ASSIGN_NARROW,
    OP_ASSIGN_I128,
    OP_ADD_I64,
    OP_SUB_I64,
    OP_ADD_I128,
    OP_FMA_I64,
    OP_MUL_I64,
    OP_MUL_MONT,
    OP_ADD_RED_DOUBLE,
    OP_RED_DOUBLE,
    OP_ADD_RED,
    OP_RED,
    OP_I128_TO_MONT,
    OP_I64_TO_MONT,
};

int64_t numel(const hc_view& v) { return v.shape[0] * v.shape[1] * v.shape[2] * v.shape[3]; }

hc_status check_view(const hc_view& v, const char* name) {
    for (int d = 0; d < 4; d++)
        if (v.shape[d] < 0) return fail(HC_ERR_SHAPE, std::string(name) + ": negative dimension");
    if (v.shape[3] > 1 && v.strides[3] != 1)
        return fail(HC_ERR_SHAPE, std::string(name) + ": dimension 3 must be contiguous (stride 1)");
    if (numel(v) > 0 && !v.ptr) return fail(HC_ERR_ARG, std::string(name) + ": null data pointer");
    return HC_OK;
}

KView kview(const hc_view& v) {
    KView k;
    k.p = (char*)v.ptr;
    k.n0 = v.shape[0], k.n1 = v.shape[1], k.n2 = v.shape[2], k.n3 = v.shape[3];
    k.s0 = v.strides[0], k.s1 = v.strides[1], k.s2 = v.strides[2];
    k.b3 = 0;
    return k;
}

/// A source view broadcast to `dst_shape` (src/hal/cpu.rs:333-346): length-1 dimensions that
/// differ from the destination get stride 0.
hc_status bview(const hc_view& src, const int64_t* dst_shape, const char* name, KView* out) {
    hc_status st = check_view(src, name);
    if (st) return st;
    *out = kview(src);
    int64_t* strides[3] = {&out->s0, &out->s1, &out->s2};
    for (int d = 0; d < 4; d++) {
        if (src.shape[d] == dst_shape[d]) continue;
        if (src.shape[d] != 1)
            return fail(HC_ERR_SHAPE, std::string("cannot broadcast dimension ") + std::to_string(d) + " of " + name +
                                          " (length " + std::to_string(src.shape[d]) + ") to length " +
                                          std::to_string(dst_shape[d]));
        if (d < 3) *strides[d] = 0;
        else out->b3 = 1;
    }
    return HC_OK;
}

hc_status kmods(const hc_modulus* mods, size_t n, int64_t rows, KMods* out) {
    if ((int64_t)n != rows) return fail(HC_ERR_SHAPE, "one modulus per RNS row (dimension 1) required");
    if (n > HC_MAX_MODS) return fail(HC_ERR_UNSUPPORTED, "too many RNS rows in one call");
    if (n && !mods) return fail(HC_ERR_ARG, "null moduli");
    for (size_t j = 0; j < n; j++) {
        out->n[j] = mods[j].n;
        out->ninv[j] = mods[j].neg_inv_n;
        out->r2[j] = mods[j].r2_mod_n;
        out->r3[j] = mods[j].r3_mod_n;
    }
    return HC_OK;
}

bool is_contiguous(const hc_view& v) {
    int64_t expect = 1;
    for (int d = 3; d >= 0; d--) {
        if (v.shape[d] > 1 && v.strides[d] != expect) return false;
        expect *= v.shape[d];
    }
    return true;
}

hc_view contiguous_view(void* p, const int64_t* shape) {
    hc_view v;
    v.ptr = p;
    for (int d = 0; d < 4; d++) v.shape[d] = shape[d];
    v.strides[3] = 1;
    v.strides[2] = shape[3];
    v.strides[1] = shape[2] * shape[3];
    v.strides[0] = shape[1] * shape[2] * shape[3];
    return v;
}

hc_status pointwise2(hc_context ctx, int op, const hc_view& dst, const hc_view& src, const hc_modulus* mods,
                     size_t nmods, bool need_mods) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st = check_view(dst, "dst");
    if (st) return st;
    KView d = kview(dst), a;
    if ((st = bview(src, dst.shape, "src", &a))) return st;
    KMods m;
    if (need_mods && (st = kmods(mods, nmods, dst.shape[1], &m))) return st;
    return launch_pointwise(ctx, op, d, a, a, m);
}

/// Host-side Montgomery constants (src/hal/mont.rs:13-33).
hc_status make_modulus(int64_t N, hc_modulus* out) {
    if (N <= 1 || (N & 1) == 0) return fail(HC_ERR_ARG, "modulus must be odd and > 1");
    uint64_t inv = (uint64_t)N;
    for (int i = 0; i < 7; i++) inv *= 2 - (uint64_t)N * inv;
    auto pmod = [N](i128 x) -> int64_t {
        i128 r = (x % (i128)N) + (i128)N;
        if (r > (i128)N) r -= N;
        return (int64_t)r;
    };
    i128 r1 = pmod((i128)1 << 64);
    out->n = N;
    out->neg_inv_n = (int64_t)(0 - inv);
    out->r2_mod_n = pmod(r1 * r1);
    out->r3_mod_n = pmod((i128)out->r2_mod_n * r1);
    return HC_OK;
}

hc_status transfer(hc_context ctx, const hc_view& v, void* host, size_t len, bool to_device, size_t esize) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st = check_view(v, to_device ? "dst" : "src");
    if (st) return st;
    if ((int64_t)len != numel(v)) return fail(HC_ERR_SHAPE, "host buffer length does not match the view");
    if (len == 0) return HC_OK;
    if (!host) return fail(HC_ERR_ARG, "null host buffer");
    cudaStream_t s = ctx->stream;
    size_t bytes = len * esize;
    if (is_contiguous(v)) {
        st = cuda_check(to_device ? cudaMemcpyAsync(v.ptr, host, bytes, cudaMemcpyHostToDevice, s)
                                  : cudaMemcpyAsync(host, v.ptr, bytes, cudaMemcpyDeviceToHost, s),
                        "import/export copy");
        if (st) return st;
        return cuda_check(cudaStreamSynchronize(s), "import/export sync");
    }
    // strided view: stage contiguously on the device and scatter / gather with a copy kernel
    void* tmp = nullptr;
    count_alloc();
    if ((st = cuda_check(cudaMallocAsync(&tmp, bytes, s), "staging allocation"))) return st;
    hc_view tv = contiguous_view(tmp, v.shape);
    int op = esize == 16 ? OP_ASSIGN_I128 : OP_ASSIGN;
    KMods dummy;
    if (to_device) {
        st = cuda_check(cudaMemcpyAsync(tmp, host, bytes, cudaMemcpyHostToDevice, s), "import copy");
        if (!st) st = launch_pointwise(ctx, op, kview(v), kview(tv), kview(tv), dummy);
    } else {
        st = launch_pointwise(ctx, op, kview(tv), kview(v), kview(v), dummy);
        if (!st) st = cuda_check(cudaMemcpyAsync(host, tmp, bytes, cudaMemcpyDeviceToHost, s), "export copy");
    }
    cudaFreeAsync(tmp, s);
    hc_status st2 = cuda_check(cudaStreamSynchronize(s), "import/export sync");
    return st ? st : st2;
}

hc_status alloc(hc_context ctx, const int64_t shape[4], size_t esize, void** out) {
    if (!ctx || !out || !shape) return fail(HC_ERR_ARG, "null argument");
    size_t n = 1;
    for (int d = 0; d < 4; d++) {
        if (shape[d] < 0) return fail(HC_ERR_SHAPE, "negative dimension");
        n *= (size_t)shape[d];
    }
    size_t bytes = n * esize;
    *out = nullptr;
    if (bytes == 0) bytes = 16;
    count_alloc();
    hc_status st = cuda_check(cudaMallocAsync(out, bytes, ctx->stream), "device allocation");
    if (st) return st;
    return cuda_check(cudaMemsetAsync(*out, 0, bytes, ctx->stream), "zero fill");
}

}  // namespace

extern "C" {

const char* hc_last_error(void) { return g_error.c_str(); }

hc_status hc_context_create(int device, hc_context* out) {
    if (!out) return fail(HC_ERR_ARG, "null output");
    hc_status st = cuda_check(cudaSetDevice(device), "cudaSetDevice");
    if (st) return st;
    auto* c = new hc_context_s();
    c->device = device;
    c->launches = 0;
    if ((st = cuda_check(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking), "stream creation"))) {
        delete c;
        return st;
    }
    c->stream = c->own;
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    int smem = 0;
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    c->smem_optin = (size_t)smem;
    *out = c;
    return HC_OK;
}

hc_status hc_context_destroy(hc_context ctx) {
    if (!ctx) return HC_OK;
    cudaStreamSynchronize(ctx->stream);
    cudaStreamDestroy(ctx->own);
    delete ctx;
    return HC_OK;
}

hc_status hc_context_set_stream(hc_context ctx, void* stream) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own;
    return HC_OK;
}
void* hc_context_stream(hc_context ctx) { return ctx ? (void*)ctx->stream : nullptr; }
hc_status hc_synchronize(hc_context ctx) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    return cuda_check(cudaStreamSynchronize(ctx->stream), "stream synchronize");
}
uint64_t hc_launch_count(hc_context ctx) { return ctx ? ctx->launches : 0; }

hc_status hc_allocate_i64(hc_context ctx, const int64_t shape[4], void** out) { return alloc(ctx, shape, 8, out); }
hc_status hc_allocate_i128(hc_context ctx, const int64_t shape[4], void** out) { return alloc(ctx, shape, 16, out); }
hc_status hc_free(hc_context ctx, void* ptr) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    if (!ptr) return HC_OK;
    return cuda_check(cudaFreeAsync(ptr, ctx->stream), "device free");
}

hc_status hc_import(hc_context ctx, hc_view dst, const int64_t* src, size_t len) {
    return transfer(ctx, dst, (void*)src, len, true, 8);
}
hc_status hc_export(hc_context ctx, hc_view src, int64_t* dst, size_t len) {
    return transfer(ctx, src, dst, len, false, 8);
}
hc_status hc_import_i128(hc_context ctx, hc_view dst, const int64_t* src, size_t len) {
    return transfer(ctx, dst, (void*)src, len, true, 16);
}
hc_status hc_export_i128(hc_context ctx, hc_view src, int64_t* dst, size_t len) {
    return transfer(ctx, src, dst, len, false, 16);
}

hc_status hc_assign(hc_context ctx, hc_view dst, hc_view src) { return pointwise2(ctx, OP_ASSIGN, dst, src, nullptr, 0, false); }
hc_status hc_assign_narrow(hc_context ctx, hc_view dst, hc_view src) {
    return pointwise2(ctx, OP_ASSIGN_NARROW, dst, src, nullptr, 0, false);
}
hc_status hc_assign_i128(hc_context ctx, hc_view dst, hc_view src) {
    return pointwise2(ctx, OP_ASSIGN_I128, dst, src, nullptr, 0, false);
}
hc_status hc_add_i64(hc_context ctx, hc_view dst, hc_view src) { return pointwise2(ctx, OP_ADD_I64, dst, src, nullptr, 0, false); }
hc_status hc_sub_i64(hc_context ctx, hc_view dst, hc_view src) { return pointwise2(ctx, OP_SUB_I64, dst, src, nullptr, 0, false); }
hc_status hc_add_i128(hc_context ctx, hc_view dst, hc_view src) {
    return pointwise2(ctx, OP_ADD_I128, dst, src, nullptr, 0, false);
}

static hc_status fma_like(hc_context ctx, int op, hc_view dst, hc_view lhs, hc_view rhs) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st = check_view(dst, "dst");
    if (st) return st;
    KView d = kview(dst), a, b;
    if ((st = bview(lhs, dst.shape, "lhs", &a))) return st;
    if ((st = bview(rhs, dst.shape, "rhs", &b))) return st;
    KMods m;
    return launch_pointwise(ctx, op, d, a, b, m);
}
hc_status hc_fma_i64(hc_context ctx, hc_view dst, hc_view lhs, hc_view rhs) { return fma_like(ctx, OP_FMA_I64, dst, lhs, rhs); }
hc_status hc_mul_i64(hc_context ctx, hc_view dst, hc_view lhs, hc_view rhs) { return fma_like(ctx, OP_MUL_I64, dst, lhs, rhs); }

hc_status hc_inner_product_i64(hc_context ctx, hc_view dst, const hc_view* lhs, const hc_view* rhs, size_t terms) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    if (terms < 1) return fail(HC_ERR_ARG, "inner_product_i64 requires at least one term");
    if (terms > HC_MAX_TERMS) return fail(HC_ERR_UNSUPPORTED, "too many inner-product terms");
    if (!lhs || !rhs) return fail(HC_ERR_ARG, "null term arrays");
    hc_status st = check_view(dst, "dst");
    if (st) return st;
    KView l[HC_MAX_TERMS], r[HC_MAX_TERMS];
    for (size_t t = 0; t < terms; t++) {
        if ((st = bview(lhs[t], dst.shape, "lhs term", &l[t]))) return st;
        if ((st = bview(rhs[t], dst.shape, "rhs term", &r[t]))) return st;
    }
    return launch_inner_product(ctx, kview(dst), l, r, (int)terms);
}

hc_status hc_matmul_i64(hc_context ctx, hc_view dst, hc_view lhs, hc_view rhs) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st;
    if ((st = check_view(dst, "dst")) || (st = check_view(lhs, "lhs")) || (st = check_view(rhs, "rhs"))) return st;
    const int64_t I = dst.shape[0], J = dst.shape[1], K = dst.shape[2], L = dst.shape[3], U = lhs.shape[2];
    if (!(lhs.shape[0] == I || lhs.shape[0] == 1)) return fail(HC_ERR_SHAPE, "matmul: lhs dimension 0");
    if (lhs.shape[1] != J || lhs.shape[3] != 1) return fail(HC_ERR_SHAPE, "matmul: lhs must have shape [I|1, J, U, 1]");
    if (!(rhs.shape[0] == I || rhs.shape[0] == 1)) return fail(HC_ERR_SHAPE, "matmul: rhs dimension 0");
    if (rhs.shape[1] != U || rhs.shape[2] != K || rhs.shape[3] != L)
        return fail(HC_ERR_SHAPE, "matmul: rhs must have shape [I|1, U, K, L]");
    if (U > 256) return fail(HC_ERR_UNSUPPORTED, "matmul: inner dimension above 256");
    KView d = kview(dst), a = kview(lhs), b = kview(rhs);
    if (lhs.shape[0] == 1) a.s0 = 0;
    if (rhs.shape[0] == 1) b.s0 = 0;
    return launch_matmul(ctx, d, a, b, U);
}

hc_status hc_create_modulus(int64_t prime, hc_modulus* out) {
    if (!out) return fail(HC_ERR_ARG, "null output");
    return make_modulus(prime, out);
}

hc_status hc_mul_mont64(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_MUL_MONT, dst, src, mods, nmods, true);
}
hc_status hc_add_red_mont64_double(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_ADD_RED_DOUBLE, dst, src, mods, nmods, true);
}
hc_status hc_red_mont64_double(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_RED_DOUBLE, dst, src, mods, nmods, true);
}
hc_status hc_add_red_mont64(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_ADD_RED, dst, src, mods, nmods, true);
}
hc_status hc_red_mont64(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_RED, dst, src, mods, nmods, true);
}
hc_status hc_i128_to_mont64(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_I128_TO_MONT, dst, src, mods, nmods, true);
}
hc_status hc_i64_to_mont64(hc_context ctx, hc_view dst, const hc_modulus* mods, size_t nmods) {
    return pointwise2(ctx, OP_I64_TO_MONT, dst, dst, mods, nmods, true);
}

hc_status hc_create_ntt_plan(hc_context ctx, const hc_modulus* modulus, const size_t* inner_shape, size_t k,
                             hc_ntt_plan* out) {
    if (!ctx || !modulus || !out || (k && !inner_shape)) return fail(HC_ERR_ARG, "null argument");
    return build_plan(ctx, modulus, inner_shape, k, out);
}
hc_status hc_destroy_ntt_plan(hc_context ctx, hc_ntt_plan plan) {
    (void)ctx;
    return destroy_plan(plan);
}

static hc_status ntt_call(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim,
                          int mode, const hc_view* mul, const hc_modulus* mods, size_t nmods) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    if (dim != HC_DIM2 && dim != HC_DIM3) return fail(HC_ERR_ARG, "dim must be 2 or 3");
    if (nplans && !plans) return fail(HC_ERR_ARG, "null plans");
    hc_status st = check_view(dst, "dst");
    if (st) return st;
    KView t = kview(dst), m = t;
    KMods km;
    if (mode & 2) {
        if ((st = bview(*mul, dst.shape, "mul", &m))) return st;
        if ((st = kmods(mods, nmods, dst.shape[1], &km))) return st;
    }
    return launch_ntt(ctx, t, plans, nplans, (int)dim, mode, m, km);
}

}  // extern "C"

namespace hc {
/// Inverse transform followed by a Montgomery product with `mul` in the epilogue of the last pass
/// (the same integers as hc_intt_mont64_dim followed by hc_mul_mont64); used by the ring layer.
hc_status intt_mul_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim,
                              hc_view mul, const hc_modulus* mods, size_t nmods) {
    return ntt_call(ctx, dst, plans, nplans, dim, 3, &mul, mods, nmods);
}

/// hc_assign(dst, src) followed by hc_ntt_mul_mont64_dim on dst, with the copy folded into the
/// transform's reads where the column kernel runs the call; used by the ring layer.
hc_status ntt_mul_mont64_dim_from(hc_context ctx, hc_view dst, hc_view src, const hc_ntt_plan* plans, size_t nplans,
                                  hc_data_dim dim, hc_view mul, const hc_modulus* mods, size_t nmods) {
    hc_status st;
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    if (nplans && !plans) return fail(HC_ERR_ARG, "null plans");
    // the column kernel reads each column whole before writing it: an exact alias is an in-place
    // call; any other overlap of the two views' address ranges takes the copy path
    auto range = [](const hc_view& v, const char** lo, const char** hi) {
        int64_t last = 0;
        for (int d = 0; d < 4; d++) last += (v.shape[d] > 0 ? v.shape[d] - 1 : 0) * (d == 3 ? 1 : v.strides[d]);
        *lo = (const char*)v.ptr;
        *hi = (const char*)v.ptr + 8 * (last + 1);
    };
    const char *dl, *dh, *sl, *sh;
    range(dst, &dl, &dh);
    range(src, &sl, &sh);
    const bool overlap = src.ptr != dst.ptr && sl < dh && dl < sh;
    if (overlap || !ntt_column_path(plans, nplans, (int)dim)) {
        if ((st = hc_assign(ctx, dst, src))) return st;
        return ntt_call(ctx, dst, plans, nplans, dim, 2, &mul, mods, nmods);
    }
    if ((st = check_view(dst, "dst")) || (st = check_view(src, "src"))) return st;
    for (int d = 0; d < 4; d++)
        if (src.shape[d] != dst.shape[d]) return fail(HC_ERR_SHAPE, "source and destination shapes differ");
    KView t = kview(dst), s = kview(src), m = t;
    KMods km;
    if ((st = bview(mul, dst.shape, "mul", &m))) return st;
    if ((st = kmods(mods, nmods, dst.shape[1], &km))) return st;
    return launch_ntt(ctx, t, plans, nplans, (int)dim, 2, m, km, &s);
}
}  // namespace hc

extern "C" {

hc_status hc_ntt_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim) {
    return ntt_call(ctx, dst, plans, nplans, dim, 0, nullptr, nullptr, 0);
}
hc_status hc_intt_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim) {
    return ntt_call(ctx, dst, plans, nplans, dim, 1, nullptr, nullptr, 0);
}
hc_status hc_ntt_mul_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim,
                                hc_view mul, const hc_modulus* mods, size_t nmods) {
    return ntt_call(ctx, dst, plans, nplans, dim, 2, &mul, mods, nmods);
}
hc_status hc_ntt_mont64(hc_context ctx, hc_view dst, const hc_ntt_plan* dim2, size_t n2, const hc_ntt_plan* dim3,
                        size_t n3) {
    hc_status st = hc_ntt_mont64_dim(ctx, dst, dim2, n2, HC_DIM2);
    return st ? st : hc_ntt_mont64_dim(ctx, dst, dim3, n3, HC_DIM3);
}
hc_status hc_intt_mont64(hc_context ctx, hc_view dst, const hc_ntt_plan* dim2, size_t n2, const hc_ntt_plan* dim3,
                         size_t n3) {
    hc_status st = hc_intt_mont64_dim(ctx, dst, dim2, n2, HC_DIM2);
    return st ? st : hc_intt_mont64_dim(ctx, dst, dim3, n3, HC_DIM3);
}

hc_status hc_bconv_correct_mont64(hc_context ctx, hc_view dst, hc_view lhs, hc_view rhs, const hc_modulus* mods,
                                  size_t nmods, size_t shift) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st;
    if ((st = check_view(dst, "dst")) || (st = check_view(lhs, "lhs")) || (st = check_view(rhs, "rhs"))) return st;
    const int64_t I = dst.shape[0], J = dst.shape[1], K = dst.shape[2], L = dst.shape[3];
    if (shift < 64 || shift >= 127) return fail(HC_ERR_ARG, "bconv_correct_mont64: shift must be in [64, 127)");
    if (lhs.shape[0] != I || lhs.shape[1] != 1 || lhs.shape[2] != K || lhs.shape[3] != L)
        return fail(HC_ERR_SHAPE, "bconv_correct_mont64: lhs must have shape [I, 1, K, L]");
    if (!(rhs.shape[0] == I || rhs.shape[0] == 1) || rhs.shape[1] != J || rhs.shape[2] != 1 || rhs.shape[3] != 1)
        return fail(HC_ERR_SHAPE, "bconv_correct_mont64: rhs must have shape [I|1, J, 1, 1]");
    KMods m;
    if ((st = kmods(mods, nmods, J, &m))) return st;
    KView a = kview(lhs), b = kview(rhs);
    if (rhs.shape[0] == 1) b.s0 = 0;
    return launch_bconv_correct(ctx, kview(dst), a, b, m, (int)shift);
}

hc_status hc_bconv_correct_pow2(hc_context ctx, hc_view dst, hc_view src, int64_t factor0, int64_t factor1,
                                size_t shift, size_t log2_modulus) {
    if (!ctx) return fail(HC_ERR_ARG, "null context");
    hc_status st;
    if ((st = check_view(dst, "dst")) || (st = check_view(src, "src"))) return st;
    if (dst.shape[1] != 1) return fail(HC_ERR_SHAPE, "bconv_correct_pow2: dst must have shape [I, 1, K, L]");
    if (src.shape[0] != dst.shape[0] || src.shape[1] != 2 || src.shape[2] != dst.shape[2] || src.shape[3] != dst.shape[3])
        return fail(HC_ERR_SHAPE, "bconv_correct_pow2: src must have shape [I, 2, K, L]");
    if (shift < 1 || shift >= 127) return fail(HC_ERR_ARG, "shift must be in [1, 127)");
    if (log2_modulus < 1 || log2_modulus > 62) return fail(HC_ERR_ARG, "log2_modulus must be in [1, 62]");
    return launch_bconv_pow2(ctx, kview(dst), kview(src), (i128)factor0, (i128)factor1, (int)shift, (int)log2_modulus, 0);
}

hc_status hc_bconv_correct_pow2_wide(hc_context ctx, hc_view dst, hc_view src, const int64_t factor0[2],
                                     const int64_t factor1[2], size_t shift, size_t log2_modulus) {
    if (!ctx || !factor0 || !factor1) return fail(HC_ERR_ARG, "null argument");
    hc_status st;
    if ((st = check_view(dst, "dst")) || (st = check_view(src, "src"))) return st;
    if (dst.shape[1] != 2) return fail(HC_ERR_SHAPE, "bconv_correct_pow2_wide: dst must have shape [I, 2, K, L]");
    if (src.shape[0] != dst.shape[0] || src.shape[1] != 3 || src.shape[2] != dst.shape[2] || src.shape[3] != dst.shape[3])
        return fail(HC_ERR_SHAPE, "bconv_correct_pow2_wide: src must have shape [I, 3, K, L]");
    if (shift < 1 || shift >= 127) return fail(HC_ERR_ARG, "shift must be in [1, 127)");
    if (log2_modulus < 1 || log2_modulus > 126) return fail(HC_ERR_ARG, "log2_modulus must be in [1, 126]");
    i128 f0 = (i128)(((u128)(uint64_t)factor0[1] << 64) | (uint64_t)factor0[0]);
    i128 f1 = (i128)(((u128)(uint64_t)factor1[1] << 64) | (uint64_t)factor1[0]);
    return launch_bconv_pow2(ctx, kview(dst), kview(src), f0, f1, (int)shift, (int)log2_modulus, 1);
}

hc_status hc_create_permutation(hc_context ctx, const size_t* inner_shape, const size_t* shifts, size_t k,
                                hc_perm_plan* out) {
    if (!ctx || !out || (k && (!inner_shape || !shifts))) return fail(HC_ERR_ARG, "null argument");
    size_t n = 1;
    for (size_t t = 0; t < k; t++) n *= inner_shape[t];
    if (n > 0xffffffffull) return fail(HC_ERR_UNSUPPORTED, "permutation too long");
    std::vector<uint32_t> perm(n);
    std::vector<size_t> idx(k, 0);
    for (size_t e = 0; e < n; e++) {
        size_t src = 0;
        for (size_t t = 0; t < k; t++) {
            size_t m = inner_shape[t];
            src = src * m + (idx[t] + m - shifts[t] % m) % m;
        }
        perm[e] = (uint32_t)src;
        for (size_t t = k; t-- > 0;) {
            if (++idx[t] < inner_shape[t]) break;
            idx[t] = 0;
        }
    }
    auto* p = new hc_perm_plan_s();
    p->len = n;
    p->dev = nullptr;
    count_alloc();
    hc_status st = cuda_check(cudaMalloc(&p->dev, n * sizeof(uint32_t) + 4), "permutation allocation");
    if (!st) st = cuda_check(cudaMemcpy(p->dev, perm.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload");
    if (st) {
        cudaFree(p->dev);
        delete p;
        return st;
    }
    *out = p;
    return HC_OK;
}
hc_status hc_destroy_permutation(hc_context ctx, hc_perm_plan plan) {
    (void)ctx;
    if (plan) {
        cudaFree(plan->dev);
        delete plan;
    }
    return HC_OK;
}
hc_status hc_permute(hc_context ctx, hc_view dst, hc_view src, hc_perm_plan plan, hc_data_dim dim) {
    if (!ctx || !plan) return fail(HC_ERR_ARG, "null argument");
    hc_status st;
    if ((st = check_view(dst, "dst")) || (st = check_view(src, "src"))) return st;
    for (int d = 0; d < 4; d++)
        if (dst.shape[d] != src.shape[d]) return fail(HC_ERR_SHAPE, "permute: dst and src shapes differ");
    if (dim != HC_DIM2 && dim != HC_DIM3) return fail(HC_ERR_ARG, "dim must be 2 or 3");
    if ((int64_t)plan->len != dst.shape[dim]) return fail(HC_ERR_SHAPE, "permutation length does not match the dimension");
    return launch_permute(ctx, kview(dst), kview(src), plan->dev, (int)dim);
}

}  // extern "C"

/*
 * halcuda.h — C ABI of the GB300 (sm_103a) ring-arithmetic backend.
 *
 * Every entry point of part 1 replaces one method of the reference's tensor HAL trait
 * `hal::Backend` (cyclosubfield-dbfv/src/hal/mod.rs:108-350), whose only implementation is
 * `hal::cpu::CpuBackend` (cyclosubfield-dbfv/src/hal/cpu.rs:553-1123). Results are bit-identical to
 * that implementation on the same inputs. Part 2 adds fused ring-level operations and a batched
 * launch API that the trait cannot express (one trait call has one shape).
 *
 * Conventions
 *  - Tensors are 4-D, row-major-strided views of device memory (`hc_view`): strides are in
 *    elements, the dimension-3 stride must be 1 (or dimension 3 has length 1). Dimension 1 is the
 *    RNS index: entry [i, j, k, l] is a residue modulo the j-th modulus of the call.
 *  - i64 tensors hold 8-byte elements; i128 tensors hold 16-byte two's-complement elements
 *    (low word first), the layout of `__int128`.
 *  - Pointwise operations broadcast source dimensions of length 1 (src/hal/mod.rs:84-90).
 *  - All operations are enqueued on the context's CUDA stream and are asynchronous, except
 *    hc_import / hc_export (and their i128 variants), which return once the host buffer may be
 *    reused (as the reference's import/export do).
 *  - Every entry point checks shapes and arguments on the host (the reference `assert!`s, with
 *    `panic = "abort"`, Cargo.toml:28) and returns a status instead; hc_last_error() describes
 *    the last failure of the calling thread.
 */
#ifndef HALCUDA_H
#define HALCUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    HC_OK = 0,
    HC_ERR_SHAPE = 1,       /* shapes / broadcasting / strides violate the method's contract */
    HC_ERR_ARG = 2,         /* other invalid argument (null pointer, bad modulus, bad shift ...) */
    HC_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    HC_ERR_OOM = 4,         /* device allocation failed */
    HC_ERR_TIMEOUT = 5,     /* a bounded wait expired */
    HC_ERR_UNSUPPORTED = 6, /* size beyond a documented implementation limit */
} hc_status;

typedef struct hc_context_s* hc_context;
typedef struct hc_ntt_plan_s* hc_ntt_plan;
typedef struct hc_perm_plan_s* hc_perm_plan;

/* A strided 4-D view of device memory. */
typedef struct {
    void* ptr;
    int64_t shape[4];
    int64_t strides[4];
} hc_view;

/* Montgomery modulus, R = 2^64 (MontgomeryModulus, src/hal/mont.rs:4-33). A plain value, like
 * the reference's `Copy` type; create it with hc_create_modulus. */
typedef struct {
    int64_t n;
    int64_t neg_inv_n;   /* -n^-1 mod 2^64 */
    int64_t r2_mod_n;    /* 2^128 mod n, in (0, n] */
    int64_t r3_mod_n;    /* 2^192 mod n, in (0, n] */
} hc_modulus;

typedef enum { HC_DIM2 = 2, HC_DIM3 = 3 } hc_data_dim; /* DataDim, src/hal/mod.rs:79-82 */

/* ---------------------------------------------------------------- context */
const char* hc_last_error(void);
hc_status hc_context_create(int device, hc_context* out);
hc_status hc_context_destroy(hc_context ctx);
/* Use `stream` (a cudaStream_t) for all further work of this context; NULL selects the
 * context's own stream. */
hc_status hc_context_set_stream(hc_context ctx, void* stream);
void* hc_context_stream(hc_context ctx);
hc_status hc_synchronize(hc_context ctx);
/* Number of kernels this context launched so far (for launch accounting). */
uint64_t hc_launch_count(hc_context ctx);

/* =============================================================================================
 * Part 1: the Backend trait
 * ============================================================================================= */

/* hal_allocate_i64 / hal_allocate_i128 (src/hal/mod.rs:120-123): zero-initialised, contiguous. */
hc_status hc_allocate_i64(hc_context ctx, const int64_t shape[4], void** out);
hc_status hc_allocate_i128(hc_context ctx, const int64_t shape[4], void** out);
hc_status hc_free(hc_context ctx, void* ptr);

/* hal_import / hal_export (src/hal/mod.rs:124-125, src/hal/cpu.rs:566-589): host buffers hold
 * the view's elements in row-major order; `len` must equal the view's element count. */
hc_status hc_import(hc_context ctx, hc_view dst, const int64_t* src, size_t len);
hc_status hc_export(hc_context ctx, hc_view src, int64_t* dst, size_t len);
/* i128 transfers (2 int64 words per element); the trait has none, tests and callers use them. */
hc_status hc_import_i128(hc_context ctx, hc_view dst, const int64_t* src, size_t len);
hc_status hc_export_i128(hc_context ctx, hc_view src, int64_t* dst, size_t len);

/* hal_assign, hal_assign_narrow, hal_assign_i128 (src/hal/mod.rs:127-139) */
hc_status hc_assign(hc_context ctx, hc_view dst, hc_view src);
hc_status hc_assign_narrow(hc_context ctx, hc_view dst, hc_view src_i128);
hc_status hc_assign_i128(hc_context ctx, hc_view dst_i128, hc_view src_i128);

/* hal_add_i64, hal_sub_i64, hal_add_i128 (src/hal/mod.rs:141-143): wrapping */
hc_status hc_add_i64(hc_context ctx, hc_view dst, hc_view src);
hc_status hc_sub_i64(hc_context ctx, hc_view dst, hc_view src);
hc_status hc_add_i128(hc_context ctx, hc_view dst_i128, hc_view src_i128);

/* hal_fma_i64 / hal_mul_i64 (src/hal/mod.rs:146-151): dst(i128) (+)= lhs * rhs */
hc_status hc_fma_i64(hc_context ctx, hc_view dst_i128, hc_view lhs, hc_view rhs);
hc_status hc_mul_i64(hc_context ctx, hc_view dst_i128, hc_view lhs, hc_view rhs);

/* hal_inner_product_i64 (src/hal/mod.rs:153-166): dst(i128) = sum_t lhs[t] * rhs[t], overwriting;
 * 1 <= terms <= 64. */
hc_status hc_inner_product_i64(hc_context ctx, hc_view dst_i128, const hc_view* lhs, const hc_view* rhs,
                               size_t terms);

/* hal_matmul_i64 (src/hal/mod.rs:168-177): dst[i,j,k,l] = sum_u lhs[i,j,u,0] * rhs[i,u,k,l];
 * lhs and rhs may broadcast dimension 0; u <= 256. */
hc_status hc_matmul_i64(hc_context ctx, hc_view dst_i128, hc_view lhs, hc_view rhs);

/* hal_create_modulus (src/hal/mod.rs:179, src/hal/mont.rs:13-33) */
hc_status hc_create_modulus(int64_t prime, hc_modulus* out);

/* hal_mul_mont64 (src/hal/mod.rs:181-183): dst = red(dst * src), `mods[j]` for row j. */
hc_status hc_mul_mont64(hc_context ctx, hc_view dst, hc_view src, const hc_modulus* mods, size_t nmods);
/* hal_add_red_mont64_double / hal_red_mont64_double (src/hal/mod.rs:185-194) */
hc_status hc_add_red_mont64_double(hc_context ctx, hc_view dst, hc_view src_i128, const hc_modulus* mods,
                                   size_t nmods);
hc_status hc_red_mont64_double(hc_context ctx, hc_view dst, hc_view src_i128, const hc_modulus* mods, size_t nmods);
/* hal_add_red_mont64 / hal_red_mont64 (src/hal/mod.rs:196-205) */
hc_status hc_add_red_mont64(hc_context ctx, hc_view dst, hc_view src_i128, const hc_modulus* mods, size_t nmods);
hc_status hc_red_mont64(hc_context ctx, hc_view dst, hc_view src_i128, const hc_modulus* mods, size_t nmods);
/* hal_i128_to_mont64 / hal_i64_to_mont64 (src/hal/mod.rs:207-213) */
hc_status hc_i128_to_mont64(hc_context ctx, hc_view dst, hc_view src_i128, const hc_modulus* mods, size_t nmods);
hc_status hc_i64_to_mont64(hc_context ctx, hc_view dst, const hc_modulus* mods, size_t nmods);

/* hal_create_ntt_plan (src/hal/mod.rs:215, src/hal/ntt.rs:561-566): the group NTT over
 * C_n0 x ... x C_n(k-1), each n_i a power of 2 or of 3. The plan's twiddle tables and its stage
 * program (the reference's data-independent reduction schedule) live in device memory. */
hc_status hc_create_ntt_plan(hc_context ctx, const hc_modulus* modulus, const size_t* inner_shape, size_t k,
                             hc_ntt_plan* out);
hc_status hc_destroy_ntt_plan(hc_context ctx, hc_ntt_plan plan);
/* hal_ntt_mont64_dim / hal_intt_mont64_dim / hal_ntt_mul_mont64_dim (src/hal/mod.rs:217-239),
 * one plan per row j; nplans == shape[1]. */
hc_status hc_ntt_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim);
hc_status hc_intt_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans, hc_data_dim dim);
hc_status hc_ntt_mul_mont64_dim(hc_context ctx, hc_view dst, const hc_ntt_plan* plans, size_t nplans,
                                hc_data_dim dim, hc_view mul, const hc_modulus* mods, size_t nmods);
/* hal_ntt_mont64 / hal_intt_mont64 (default methods, src/hal/mod.rs:241-250) */
hc_status hc_ntt_mont64(hc_context ctx, hc_view dst, const hc_ntt_plan* dim2, size_t n2, const hc_ntt_plan* dim3,
                        size_t n3);
hc_status hc_intt_mont64(hc_context ctx, hc_view dst, const hc_ntt_plan* dim2, size_t n2, const hc_ntt_plan* dim3,
                         size_t n3);

/* hal_bconv_correct_mont64 (src/hal/mod.rs:252-270):
 * dst[i,j,k,l] += red(rounddiv(lhs[i,0,k,l], 2^shift) * rhs[i,j,0,0]), 64 <= shift < 127 */
hc_status hc_bconv_correct_mont64(hc_context ctx, hc_view dst, hc_view lhs_i128, hc_view rhs, const hc_modulus* mods,
                                  size_t nmods, size_t shift);
/* hal_bconv_correct_pow2 (src/hal/mod.rs:272-297) */
hc_status hc_bconv_correct_pow2(hc_context ctx, hc_view dst, hc_view src_i128, int64_t factor0, int64_t factor1,
                                size_t shift, size_t log2_modulus);
/* hal_bconv_correct_pow2_wide (src/hal/mod.rs:299-338); the i128 factors as (low, high) words */
hc_status hc_bconv_correct_pow2_wide(hc_context ctx, hc_view dst, hc_view src_i128, const int64_t factor0[2],
                                     const int64_t factor1[2], size_t shift, size_t log2_modulus);

/* hal_create_permutation / hal_permute (src/hal/mod.rs:340-349, src/hal/cpu.rs:1059-1122) */
hc_status hc_create_permutation(hc_context ctx, const size_t* inner_shape, const size_t* shifts, size_t k,
                                hc_perm_plan* out);
hc_status hc_destroy_permutation(hc_context ctx, hc_perm_plan plan);
hc_status hc_permute(hc_context ctx, hc_view dst, hc_view src, hc_perm_plan plan, hc_data_dim dim);

/* =============================================================================================
 * Runtime utilities (no trait counterpart): pinned host memory and asynchronous copies for
 * streaming keys and requests, CUDA events for timing, free-memory queries for admission.
 * ============================================================================================= */
typedef enum { HC_H2D = 0, HC_D2H = 1, HC_D2D = 2 } hc_copy_kind;
typedef struct hc_event_s* hc_event;

hc_status hc_host_alloc(size_t bytes, void** out); /* page-locked host memory */
hc_status hc_host_free(void* ptr);
hc_status hc_memcpy_async(hc_context ctx, void* dst, const void* src, size_t bytes, hc_copy_kind kind);
hc_status hc_memset_async(hc_context ctx, void* dst, int value, size_t bytes);
hc_status hc_event_create(hc_event* out);
hc_status hc_event_destroy(hc_event ev);
hc_status hc_event_record(hc_context ctx, hc_event ev);
/* Work issued to the context's current stream after this call starts only once the work recorded
 * before `ev` has completed (a device-side dependency; the host does not block). */
hc_status hc_stream_wait_event(hc_context ctx, hc_event ev);
/* Extra streams for concurrent work on one context: create, select with hc_context_set_stream
 * (NULL selects the context's own stream again), destroy after their work is done. */
hc_status hc_stream_create(void** out);
hc_status hc_stream_destroy(void* stream);
/* Non-blocking: *done = 1 once all work recorded before the event has completed, else 0. */
hc_status hc_event_query(hc_event ev, int* done);
/* Milliseconds between two recorded events; waits for `end` (bounded by `timeout_ms`, then
 * HC_ERR_TIMEOUT; timeout_ms <= 0 waits without bound). */
hc_status hc_event_elapsed_ms(hc_event start, hc_event end, double timeout_ms, float* ms);
hc_status hc_device_memory(hc_context ctx, size_t* free_bytes, size_t* total_bytes);
/* Device-memory bookkeeping (no trait counterpart), for callers that budget HBM and for tests that
 * a call allocates nothing: out[0] = allocation calls this library has made in the process (device
 * and pinned host, every kind), out[1] / out[2] = bytes in use / high-water mark of the device's
 * default memory pool, from which the library's stream-ordered allocations come. reset_high != 0
 * first resets the high-water mark to the bytes in use. */
hc_status hc_memory_stats(hc_context ctx, int reset_high, uint64_t out[3]);
/* Measurement utility (no reference counterpart): the GPU's rate of the transforms' exact 64-bit
 * Barrett product, from a register-only kernel on the context's stream (about a millisecond;
 * synchronises the stream). The integer-pipe roofline denominator of the compute-bound NTTs. */
hc_status hc_barrett_peak(hc_context ctx, double* products_per_s);
/* Measurement utility (no reference counterpart): the GPU's int8 tensor-core rate in
 * multiply-adds per second, from a register-only kernel of warp-level s8 x s8 -> s32 MMAs (the only
 * int8 tensor instruction sm_103a has; about a millisecond; synchronises the stream). The
 * denominator an int8 limb-split base conversion would be measured against. */
hc_status hc_int8_mma_peak(hc_context ctx, double* macs_per_s);

/* CUDA-graph capture of a sequence of calls on the context's stream (for launch-bound loops):
 * every call between begin and end is recorded, not executed; hc_graph_launch replays it. The
 * recorded calls must not synchronise with the host (hc_import / hc_export and first-use
 * set-up of ring caches do; run one uncaptured call first). Tensors allocated inside the capture
 * are graph-owned and released when the replay finishes. */
typedef struct hc_graph_s* hc_graph;
hc_status hc_graph_begin_capture(hc_context ctx);
hc_status hc_graph_end_capture(hc_context ctx, hc_graph* out);
hc_status hc_graph_launch(hc_context ctx, hc_graph graph);
hc_status hc_graph_destroy(hc_graph graph);

#ifdef __cplusplus
}
#endif

#endif /* HALCUDA_H */

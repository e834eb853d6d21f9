// ORACLE — test infrastructure only (see arith.hpp). Restates the lazy group NTT of the
// reference line by line, including its data-independent bound tracking:
//   reduce_pass        cyclosubfield-dbfv/src/hal/ntt.rs:164-173
//   LazyFactorNTT      cyclosubfield-dbfv/src/hal/ntt.rs:189-538
//   CpuNTTPlan         cyclosubfield-dbfv/src/hal/ntt.rs:549-658
#pragma once
#include <vector>

#include "arith.hpp"

namespace oracle {

/// src/hal/ntt.rs:164-173
inline void reduce_pass(BarrettMul one, int64_t n, int64_t* data, size_t elem_stride, size_t len, size_t vec_len) {
    for (size_t i = 0; i < len; i++)
        for (size_t l = 0; l < vec_len; l++) {
            int64_t* x = data + i * elem_stride + l;
            *x = one.mul(*x, n);
        }
}

inline int64_t reduce_if(bool reduce, BarrettMul mul, int64_t n, int64_t x) { return reduce ? mul.mul(x, n) : x; }

/// One cyclic factor `C_len`, len a power of 2 or 3 (src/hal/ntt.rs:189-538).
struct LazyFactorNTT {
    bool radix2;
    int64_t n;
    BarrettMul one;
    size_t len;
    std::vector<std::vector<BarrettMul>> twiddles;
    std::vector<std::vector<BarrettMul>> inv_twiddles;
    BarrettMul zeta{0, 0}, zeta2{0, 0};

    /// src/hal/ntt.rs:216-281
    static LazyFactorNTT create(int64_t n, size_t len) {
        LazyFactorNTT f;
        f.n = n;
        f.len = len;
        if (is_power_of_two(len)) {
            ORACLE_ASSERT(len >= 2, "factor length");
            ORACLE_ASSERT(2 * (u128)n <= I64_MAX_U, "modulus too large for lazy radix-2 butterflies");
            f.radix2 = true;
            f.one = BarrettMul::create(1, n);
            int64_t root = find_root_of_unity(n, len);
            int64_t inv_root = pow_mod(root, len - 1, n);
            std::vector<size_t> exps{0};
            while (exps.size() < len) {
                std::vector<BarrettMul> tw, itw;
                for (size_t e : exps) {
                    tw.push_back(BarrettMul::create(pow_mod(root, e / 2, n), n));
                    itw.push_back(BarrettMul::create(pow_mod(inv_root, e / 2, n), n));
                }
                f.twiddles.push_back(tw);
                f.inv_twiddles.push_back(itw);
                std::vector<size_t> next;
                for (size_t e : exps) {
                    next.push_back(e / 2);
                    next.push_back(e / 2 + len / 2);
                }
                exps = next;
            }
        } else {
            size_t l = len;
            while (l > 1) {
                ORACLE_ASSERT(l % 3 == 0, "NTT length must be a power of 2 or a power of 3");
                l /= 3;
            }
            ORACLE_ASSERT(len >= 3, "factor length");
            ORACLE_ASSERT(3 * (u128)n <= I64_MAX_U, "modulus too large for lazy radix-3 butterflies");
            f.radix2 = false;
            f.one = BarrettMul::create(1, n);
            int64_t root = find_root_of_unity(n, len);
            int64_t inv_root = pow_mod(root, len - 1, n);
            int64_t zeta_plain = pow_mod(root, len / 3, n);
            int64_t zeta2_plain = mul_mod(zeta_plain, zeta_plain, n);
            std::vector<size_t> exps{0};
            while (exps.size() < len) {
                std::vector<BarrettMul> tw, itw;
                for (size_t e : exps) {
                    int64_t v = pow_mod(root, e / 3, n);
                    int64_t v_sqr = mul_mod(v, v, n);
                    tw.push_back(BarrettMul::create(v, n));
                    tw.push_back(BarrettMul::create(mul_mod(zeta_plain, v, n), n));
                    tw.push_back(BarrettMul::create(mul_mod(zeta2_plain, v, n), n));
                    tw.push_back(BarrettMul::create(v_sqr, n));
                    tw.push_back(BarrettMul::create(mul_mod(zeta_plain, v_sqr, n), n));
                    tw.push_back(BarrettMul::create(mul_mod(zeta2_plain, v_sqr, n), n));
                    int64_t v_inv = pow_mod(inv_root, e / 3, n);
                    itw.push_back(BarrettMul::create(v_inv, n));
                    itw.push_back(BarrettMul::create(mul_mod(v_inv, v_inv, n), n));
                }
                f.twiddles.push_back(tw);
                f.inv_twiddles.push_back(itw);
                std::vector<size_t> next;
                for (size_t e : exps) {
                    next.push_back(e / 3);
                    next.push_back(e / 3 + len / 3);
                    next.push_back(e / 3 + 2 * (len / 3));
                }
                exps = next;
            }
            f.zeta = BarrettMul::create(zeta_plain, n);
            f.zeta2 = BarrettMul::create(zeta2_plain, n);
        }
        return f;
    }

    /// src/hal/ntt.rs:301-414
    u128 forward(int64_t* data, size_t elem_stride, size_t vec_len, u128 in_bound, bool reduce_output) const {
        u128 bound = in_bound;
        if (radix2) {
            size_t stage_len = len;
            for (size_t s = 0; s < twiddles.size(); s++) {
                const auto& stage_twiddles = twiddles[s];
                bool fuse = reduce_output && s + 1 == twiddles.size();
                if (bound + (u128)n > I64_MAX_U) {
                    reduce_pass(one, n, data, elem_stride, len, vec_len);
                    bound = (u128)n;
                }
                bool skip_ok = 2 * bound <= I64_MAX_U;
                u128 new_bound = fuse ? (u128)n : (skip_ok ? 2 * bound : bound + (u128)n);
                size_t half = stage_len / 2;
                for (size_t block = 0, block_start = 0; block_start < len; block++, block_start += stage_len) {
                    BarrettMul v = stage_twiddles[block];
                    bool skip = skip_ok && v.is_one();
                    for (size_t j = 0; j < half; j++) {
                        int64_t* x = data + (block_start + j) * elem_stride;
                        int64_t* y = data + (block_start + j + half) * elem_stride;
                        for (size_t l = 0; l < vec_len; l++) {
                            int64_t a = x[l];
                            int64_t t = skip ? y[l] : v.mul(y[l], n);
                            x[l] = reduce_if(fuse, one, n, wadd(a, t));
                            y[l] = reduce_if(fuse, one, n, wsub(a, t));
                        }
                    }
                }
                bound = new_bound;
                stage_len = half;
            }
        } else {
            size_t stage_len = len;
            for (size_t s = 0; s < twiddles.size(); s++) {
                const auto& stage_twiddles = twiddles[s];
                bool fuse = reduce_output && s + 1 == twiddles.size();
                if (bound + 2 * (u128)n > I64_MAX_U) {
                    reduce_pass(one, n, data, elem_stride, len, vec_len);
                    bound = (u128)n;
                }
                bool skip_ok = 3 * bound <= I64_MAX_U;
                u128 new_bound = fuse ? (u128)n : (skip_ok ? 3 * bound : bound + 2 * (u128)n);
                size_t third = stage_len / 3;
                for (size_t block = 0, block_start = 0; block_start < len; block++, block_start += stage_len) {
                    BarrettMul w_b = stage_twiddles[6 * block], w_bz = stage_twiddles[6 * block + 1],
                               w_bzz = stage_twiddles[6 * block + 2], w_c = stage_twiddles[6 * block + 3],
                               w_cz = stage_twiddles[6 * block + 4], w_czz = stage_twiddles[6 * block + 5];
                    bool skip = skip_ok && w_b.is_one();
                    for (size_t j = 0; j < third; j++) {
                        int64_t* x = data + (block_start + j) * elem_stride;
                        int64_t* y = data + (block_start + j + third) * elem_stride;
                        int64_t* z = data + (block_start + j + 2 * third) * elem_stride;
                        for (size_t l = 0; l < vec_len; l++) {
                            int64_t a = x[l], b = y[l], c = z[l];
                            int64_t t_b = skip ? b : w_b.mul(b, n);
                            int64_t t_bz = w_bz.mul(b, n);
                            int64_t t_bzz = w_bzz.mul(b, n);
                            int64_t t_c = skip ? c : w_c.mul(c, n);
                            int64_t t_cz = w_cz.mul(c, n);
                            int64_t t_czz = w_czz.mul(c, n);
                            x[l] = reduce_if(fuse, one, n, wadd(wadd(a, t_b), t_c));
                            y[l] = reduce_if(fuse, one, n, wadd(wadd(a, t_bz), t_czz));
                            z[l] = reduce_if(fuse, one, n, wadd(wadd(a, t_bzz), t_cz));
                        }
                    }
                }
                bound = new_bound;
                stage_len = third;
            }
        }
        return bound;
    }

    /// src/hal/ntt.rs:427-537. `final_scale` is applied when `has_scale` is set.
    u128 backward(int64_t* data, size_t elem_stride, size_t vec_len, u128 in_bound, bool has_scale,
                  BarrettMul final_scale) const {
        u128 bound = in_bound;
        if (radix2) {
            for (size_t si = inv_twiddles.size(); si-- > 0;) {
                const auto& stage_twiddles = inv_twiddles[si];
                bool fused_scale = has_scale && si == 0;
                if (2 * bound > I64_MAX_U) {
                    reduce_pass(one, n, data, elem_stride, len, vec_len);
                    bound = (u128)n;
                }
                bound = fused_scale ? (u128)n : 2 * bound;
                size_t stage_len = len >> si;
                size_t half = stage_len / 2;
                for (size_t block = 0, block_start = 0; block_start < len; block++, block_start += stage_len) {
                    bool fuse;
                    BarrettMul y_mul;
                    if (fused_scale) {
                        ORACLE_ASSERT(stage_twiddles[block].z == 1, "fused stage twiddle");
                        fuse = true;
                        y_mul = final_scale;
                    } else {
                        fuse = false;
                        y_mul = stage_twiddles[block];
                    }
                    bool skip = !fuse && y_mul.is_one();
                    for (size_t j = 0; j < half; j++) {
                        int64_t* x = data + (block_start + j) * elem_stride;
                        int64_t* y = data + (block_start + j + half) * elem_stride;
                        for (size_t l = 0; l < vec_len; l++) {
                            int64_t y0 = x[l], y1 = y[l];
                            x[l] = reduce_if(fuse, y_mul, n, wadd(y0, y1));
                            y[l] = skip ? wsub(y0, y1) : y_mul.mul(wsub(y0, y1), n);
                        }
                    }
                }
            }
        } else {
            for (size_t si = inv_twiddles.size(); si-- > 0;) {
                const auto& stage_twiddles = inv_twiddles[si];
                bool fused_scale = has_scale && si == 0;
                if (3 * bound > I64_MAX_U) {
                    reduce_pass(one, n, data, elem_stride, len, vec_len);
                    bound = (u128)n;
                }
                bound = fused_scale ? (u128)n : 3 * bound;
                size_t stage_len = len;
                for (size_t k = 0; k < si; k++) stage_len /= 3;
                size_t third = stage_len / 3;
                for (size_t block = 0, block_start = 0; block_start < len; block++, block_start += stage_len) {
                    bool fuse;
                    BarrettMul y_mul, z_mul;
                    if (fused_scale) {
                        ORACLE_ASSERT(stage_twiddles[2 * block].z == 1 && stage_twiddles[2 * block + 1].z == 1,
                                      "fused stage twiddle");
                        fuse = true;
                        y_mul = final_scale;
                        z_mul = final_scale;
                    } else {
                        fuse = false;
                        y_mul = stage_twiddles[2 * block];
                        z_mul = stage_twiddles[2 * block + 1];
                    }
                    bool skip = !fuse && y_mul.is_one();
                    for (size_t j = 0; j < third; j++) {
                        int64_t* x = data + (block_start + j) * elem_stride;
                        int64_t* y = data + (block_start + j + third) * elem_stride;
                        int64_t* z = data + (block_start + j + 2 * third) * elem_stride;
                        for (size_t l = 0; l < vec_len; l++) {
                            int64_t y0 = x[l], y1 = y[l], y2 = z[l];
                            int64_t y1z = zeta.mul(y1, n);
                            int64_t y1zz = zeta2.mul(y1, n);
                            int64_t y2z = zeta.mul(y2, n);
                            int64_t y2zz = zeta2.mul(y2, n);
                            x[l] = reduce_if(fuse, y_mul, n, wadd(wadd(y0, y1), y2));
                            int64_t sy = wadd(wadd(y0, y1zz), y2z);
                            int64_t sz = wadd(wadd(y0, y1z), y2zz);
                            y[l] = skip ? sy : y_mul.mul(sy, n);
                            z[l] = skip ? sz : z_mul.mul(sz, n);
                        }
                    }
                }
            }
        }
        return bound;
    }
};

/// The multi-factor group NTT for one modulus (src/hal/ntt.rs:549-658).
struct CpuNTTPlan {
    int64_t n;
    std::vector<LazyFactorNTT> factors;
    size_t len;
    BarrettMul inv_len;
    BarrettMul one;

    /// src/hal/ntt.rs:561-566
    static CpuNTTPlan create(int64_t n, const std::vector<size_t>& inner_shape) {
        CpuNTTPlan p;
        p.n = n;
        p.len = 1;
        for (size_t l : inner_shape) {
            if (l > 1) p.factors.push_back(LazyFactorNTT::create(n, l));
            p.len *= l;
        }
        int64_t inv_len = pow_mod((int64_t)p.len, (uint64_t)(n - 2), n);
        p.inv_len = BarrettMul::create(inv_len, n);
        p.one = BarrettMul::create(1, n);
        return p;
    }

    /// src/hal/ntt.rs:581-657
    void apply(int64_t* data, size_t elem_stride, size_t vec_len, bool inverse, bool reduce_output) const {
        u128 bound = 2 * (u128)n;
        size_t suffix_len = 1;
        for (const auto& f : factors) suffix_len *= f.len;
        size_t prefix_len = 1;
        for (size_t fi = 0; fi < factors.size(); fi++) {
            const LazyFactorNTT& factor = factors[fi];
            bool is_last_factor = fi + 1 == factors.size();
            bool fuse_forward = is_last_factor && reduce_output;
            suffix_len /= factor.len;
            u128 new_bound = bound;
            if (vec_len == elem_stride) {
                size_t inner = suffix_len * elem_stride;
                for (size_t prefix = 0; prefix < prefix_len; prefix++) {
                    int64_t* block = data + prefix * factor.len * inner;
                    new_bound = inverse ? factor.backward(block, inner, inner, bound, is_last_factor, inv_len)
                                        : factor.forward(block, inner, inner, bound, fuse_forward);
                }
            } else {
                for (size_t prefix = 0; prefix < prefix_len; prefix++)
                    for (size_t suffix = 0; suffix < suffix_len; suffix++) {
                        size_t offset = (prefix * factor.len * suffix_len + suffix) * elem_stride;
                        new_bound = inverse ? factor.backward(data + offset, suffix_len * elem_stride, vec_len,
                                                              bound, is_last_factor, inv_len)
                                            : factor.forward(data + offset, suffix_len * elem_stride, vec_len,
                                                             bound, fuse_forward);
                    }
            }
            prefix_len *= factor.len;
            bound = new_bound;
        }
        ORACLE_ASSERT(bound <= I64_MAX_U, "NTT output bound");
        if (factors.empty()) {
            if (inverse || reduce_output) {
                BarrettMul final_mul = inverse ? inv_len : one;
                for (size_t i = 0; i < len; i++)
                    for (size_t l = 0; l < vec_len; l++) {
                        int64_t* x = data + i * elem_stride + l;
                        *x = final_mul.mul(*x, n);
                    }
            }
        }
    }
};

}  // namespace oracle

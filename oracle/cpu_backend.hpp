// ORACLE — test infrastructure only (see arith.hpp). Restates `hal::cpu::CpuBackend`
// (cyclosubfield-dbfv/src/hal/cpu.rs) over strided 4-D views whose dimension-3 stride is 1:
//   views / slicing / split            src/hal/cpu.rs:137-327
//   broadcast_strides, line iteration  src/hal/cpu.rs:333-474
//   ntt_dim_impl, mul_mont64_impl      src/hal/cpu.rs:494-550
//   the 30 Backend methods             src/hal/cpu.rs:553-1123 (trait: src/hal/mod.rs:108-350)
#pragma once
#include <array>
#include <cstring>
#include <vector>

#include "ntt.hpp"

namespace oracle {

typedef std::array<size_t, 4> Shape;

inline Shape strides_for(Shape s) { return Shape{s[1] * s[2] * s[3], s[2] * s[3], s[3], 1}; }

/// A strided view (src/hal/cpu.rs:187-205); `ptr` addresses element [0,0,0,0].
template <typename T>
struct View {
    T* ptr;
    Shape shape;
    Shape strides;

    T* line(size_t i, size_t j, size_t k) const { return ptr + i * strides[0] + j * strides[1] + k * strides[2]; }
    T& at(size_t i, size_t j, size_t k, size_t l) const { return line(i, j, k)[l * strides[3]]; }
    size_t numel() const { return shape[0] * shape[1] * shape[2] * shape[3]; }

    /// src/hal/cpu.rs:66-80: ranges [start, end) per dimension.
    View slice(size_t s0, size_t e0, size_t s1, size_t e1, size_t s2, size_t e2, size_t s3, size_t e3) const {
        ORACLE_ASSERT(s0 <= e0 && e0 <= shape[0] && s1 <= e1 && e1 <= shape[1] && s2 <= e2 && e2 <= shape[2] &&
                          s3 <= e3 && e3 <= shape[3],
                      "slice bounds invalid");
        View v = *this;
        v.ptr = ptr + s0 * strides[0] + s1 * strides[1] + s2 * strides[2] + s3 * strides[3];
        v.shape = Shape{e0 - s0, e1 - s1, e2 - s2, e3 - s3};
        return v;
    }
    View rows(size_t s, size_t e) const { return slice(s, e, 0, shape[1], 0, shape[2], 0, shape[3]); }
    View base_range(size_t s, size_t e) const { return slice(0, shape[0], s, e, 0, shape[2], 0, shape[3]); }
};

/// An owned contiguous row-major tensor (src/hal/cpu.rs:137-185).
template <typename T>
struct Tensor {
    std::vector<T> data;
    Shape shape{0, 0, 0, 0};
    Tensor() {}
    explicit Tensor(Shape s) : data(s[0] * s[1] * s[2] * s[3], T(0)), shape(s) {}
    View<T> view() { return View<T>{data.data(), shape, strides_for(shape)}; }
    View<T> view() const { return View<T>{const_cast<T*>(data.data()), shape, strides_for(shape)}; }
};

/// src/hal/cpu.rs:333-346
inline Shape broadcast_strides(Shape src_shape, Shape src_strides, Shape dst_shape) {
    Shape s = src_strides;
    for (int d = 0; d < 4; d++)
        if (src_shape[d] != dst_shape[d]) {
            ORACLE_ASSERT(src_shape[d] == 1, "cannot broadcast dimension");
            s[d] = 0;
        }
    return s;
}

template <typename T, typename F>
void for_each_line1(const View<T>& dst, F f) {
    for (size_t i = 0; i < dst.shape[0]; i++)
        for (size_t j = 0; j < dst.shape[1]; j++)
            for (size_t k = 0; k < dst.shape[2]; k++) f(j, dst.line(i, j, k));
}

/// src/hal/cpu.rs:364-387 combined with bin_line (:425-436): f(j, dst_elem&, src_elem).
template <typename T, typename S, typename F>
void pointwise2(const View<T>& dst, const View<S>& src, F f) {
    Shape ss = broadcast_strides(src.shape, src.strides, dst.shape);
    bool sb = src.shape[3] != dst.shape[3];
    for (size_t i = 0; i < dst.shape[0]; i++)
        for (size_t j = 0; j < dst.shape[1]; j++)
            for (size_t k = 0; k < dst.shape[2]; k++) {
                T* dl = dst.line(i, j, k);
                const S* sl = src.ptr + i * ss[0] + j * ss[1] + k * ss[2];
                for (size_t l = 0; l < dst.shape[3]; l++) f(j, dl[l], sl[sb ? 0 : l]);
            }
}

/// src/hal/cpu.rs:390-474: f(dst_elem&, lhs_elem, rhs_elem).
template <typename T, typename A, typename B, typename F>
void pointwise3(const View<T>& dst, const View<A>& lhs, const View<B>& rhs, F f) {
    Shape ls = broadcast_strides(lhs.shape, lhs.strides, dst.shape);
    Shape rs = broadcast_strides(rhs.shape, rhs.strides, dst.shape);
    bool lb = lhs.shape[3] != dst.shape[3], rb = rhs.shape[3] != dst.shape[3];
    for (size_t i = 0; i < dst.shape[0]; i++)
        for (size_t j = 0; j < dst.shape[1]; j++)
            for (size_t k = 0; k < dst.shape[2]; k++) {
                T* dl = dst.line(i, j, k);
                const A* ll = lhs.ptr + i * ls[0] + j * ls[1] + k * ls[2];
                const B* rl = rhs.ptr + i * rs[0] + j * rs[1] + k * rs[2];
                for (size_t l = 0; l < dst.shape[3]; l++) f(dl[l], ll[lb ? 0 : l], rl[rb ? 0 : l]);
            }
}

/// `dst[e] = src[perm[e]]` (src/hal/cpu.rs:480-485)
struct CpuPermutationPlan {
    size_t len;
    std::vector<uint32_t> perm;
};

enum class DataDim { Dim2 = 2, Dim3 = 3 };

typedef View<int64_t> V64;
typedef View<i128> V128;

/// The CPU backend (src/hal/cpu.rs:489-1123). Stateless, like the reference.
struct CpuBackend {
    // ---- allocation and transfer (src/hal/cpu.rs:560-589) ----
    Tensor<int64_t> hal_allocate_i64(Shape s) const { return Tensor<int64_t>(s); }
    Tensor<i128> hal_allocate_i128(Shape s) const { return Tensor<i128>(s); }

    void hal_import(V64 dst, const int64_t* src, size_t len) const {
        ORACLE_ASSERT(len == dst.numel(), "import length");
        size_t pos = 0;
        for_each_line1(dst, [&](size_t, int64_t* line) {
            std::memcpy(line, src + pos, dst.shape[3] * sizeof(int64_t));
            pos += dst.shape[3];
        });
    }
    void hal_export(V64 src, int64_t* dst, size_t len) const {
        ORACLE_ASSERT(len == src.numel(), "export length");
        size_t pos = 0;
        for_each_line1(src, [&](size_t, int64_t* line) {
            std::memcpy(dst + pos, line, src.shape[3] * sizeof(int64_t));
            pos += src.shape[3];
        });
    }

    // ---- copies (src/hal/cpu.rs:591-631) ----
    void hal_assign(V64 dst, V64 src) const {
        pointwise2(dst, src, [](size_t, int64_t& d, int64_t s) { d = s; });
    }
    void hal_assign_narrow(V64 dst, V128 src) const {
        pointwise2(dst, src, [](size_t, int64_t& d, i128 s) { d = (int64_t)s; });
    }
    void hal_assign_i128(V128 dst, V128 src) const {
        pointwise2(dst, src, [](size_t, i128& d, i128 s) { d = s; });
    }

    // ---- integer arithmetic (src/hal/cpu.rs:633-818) ----
    void hal_add_i64(V64 dst, V64 src) const {
        pointwise2(dst, src, [](size_t, int64_t& d, int64_t s) { d = wadd(d, s); });
    }
    void hal_add_i128(V128 dst, V128 src) const {
        pointwise2(dst, src, [](size_t, i128& d, i128 s) { d = wadd128(d, s); });
    }
    void hal_sub_i64(V64 dst, V64 src) const {
        pointwise2(dst, src, [](size_t, int64_t& d, int64_t s) { d = wsub(d, s); });
    }
    void hal_fma_i64(V128 dst, V64 lhs, V64 rhs) const {
        pointwise3(dst, lhs, rhs, [](i128& d, int64_t l, int64_t r) { d = wadd128(d, (i128)l * (i128)r); });
    }
    void hal_mul_i64(V128 dst, V64 lhs, V64 rhs) const {
        pointwise3(dst, lhs, rhs, [](i128& d, int64_t l, int64_t r) { d = (i128)l * (i128)r; });
    }
    /// src/hal/cpu.rs:707-788: the 256-wide tiling does not change any result (each tile sums the
    /// terms in order), so the terms are accumulated per element in order.
    void hal_inner_product_i64(V128 dst, const std::vector<V64>& lhs, const std::vector<V64>& rhs) const {
        ORACLE_ASSERT(lhs.size() == rhs.size() && lhs.size() >= 1, "inner_product_i64 requires at least one term");
        for (size_t t = 0; t < lhs.size(); t++) {
            if (t == 0) hal_mul_i64(dst, lhs[0], rhs[0]);
            else hal_fma_i64(dst, lhs[t], rhs[t]);
        }
    }
    /// src/hal/cpu.rs:791-818
    void hal_matmul_i64(V128 dst, V64 lhs, V64 rhs) const {
        size_t i_len = dst.shape[0], j_len = dst.shape[1], k_len = dst.shape[2], l_len = dst.shape[3];
        size_t u_len = lhs.shape[2];
        ORACLE_ASSERT(lhs.shape[0] == i_len || lhs.shape[0] == 1, "matmul lhs dim 0");
        ORACLE_ASSERT(lhs.shape[1] == j_len && lhs.shape[3] == 1, "matmul lhs shape");
        ORACLE_ASSERT(rhs.shape[0] == i_len || rhs.shape[0] == 1, "matmul rhs dim 0");
        ORACLE_ASSERT(rhs.shape[1] == u_len && rhs.shape[2] == k_len && rhs.shape[3] == l_len, "matmul rhs shape");
        for (size_t i = 0; i < i_len; i++) {
            size_t li = lhs.shape[0] == 1 ? 0 : i, ri = rhs.shape[0] == 1 ? 0 : i;
            for (size_t j = 0; j < j_len; j++)
                for (size_t k = 0; k < k_len; k++) {
                    i128* dl = dst.line(i, j, k);
                    for (size_t l = 0; l < l_len; l++) dl[l] = 0;
                    for (size_t u = 0; u < u_len; u++) {
                        i128 c = (i128)lhs.at(li, j, u, 0);
                        if (c == 0) continue;
                        const int64_t* rl = rhs.line(ri, u, k);
                        for (size_t l = 0; l < l_len; l++) dl[l] = wadd128(dl[l], wmul128(c, (i128)rl[l]));
                    }
                }
        }
    }

    // ---- Montgomery arithmetic (src/hal/cpu.rs:820-916) ----
    MontgomeryModulus hal_create_modulus(int64_t prime) const { return MontgomeryModulus::create(prime); }

    void hal_mul_mont64(V64 dst, V64 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, int64_t s) { d = mods[j].red128((i128)d * (i128)s); });
    }
    void hal_add_red_mont64_double(V64 dst, V128 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, i128 s) { d = wadd(d, mods[j].double_red128(s)); });
    }
    void hal_red_mont64_double(V64 dst, V128 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, i128 s) { d = mods[j].double_red128(s); });
    }
    void hal_add_red_mont64(V64 dst, V128 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, i128 s) { d = wadd(d, mods[j].red128(s)); });
    }
    void hal_red_mont64(V64 dst, V128 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, i128 s) { d = mods[j].red128(s); });
    }
    void hal_i128_to_mont64(V64 dst, V128 src, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        pointwise2(dst, src, [&](size_t j, int64_t& d, i128 s) { d = mods[j].to_mont128(s); });
    }
    void hal_i64_to_mont64(V64 dst, const std::vector<MontgomeryModulus>& mods) const {
        ORACLE_ASSERT(mods.size() == dst.shape[1], "moduli count");
        for_each_line1(dst, [&](size_t j, int64_t* line) {
            for (size_t l = 0; l < dst.shape[3]; l++) line[l] = mods[j].to_mont64(line[l]);
        });
    }

    // ---- NTT (src/hal/cpu.rs:494-534, :918-948) ----
    CpuNTTPlan hal_create_ntt_plan(const MontgomeryModulus& m, const std::vector<size_t>& inner_shape) const {
        return CpuNTTPlan::create(m.N, inner_shape);
    }
    void ntt_dim_impl(V64 dst, const std::vector<const CpuNTTPlan*>& ntt, DataDim dim, bool inverse,
                      bool reduce_output) const {
        ORACLE_ASSERT(ntt.size() == dst.shape[1], "plan count");
        if (dim == DataDim::Dim2) {
            for (auto p : ntt) ORACLE_ASSERT(p->len == dst.shape[2], "plan length (dim 2)");
            for (size_t i = 0; i < dst.shape[0]; i++)
                for (size_t j = 0; j < dst.shape[1]; j++)
                    ntt[j]->apply(dst.ptr + i * dst.strides[0] + j * dst.strides[1], dst.strides[2], dst.shape[3],
                                  inverse, reduce_output);
        } else {
            for (auto p : ntt) ORACLE_ASSERT(p->len == dst.shape[3], "plan length (dim 3)");
            for (size_t i = 0; i < dst.shape[0]; i++)
                for (size_t j = 0; j < dst.shape[1]; j++)
                    for (size_t k = 0; k < dst.shape[2]; k++)
                        ntt[j]->apply(dst.line(i, j, k), 1, 1, inverse, reduce_output);
        }
    }
    void hal_ntt_mont64_dim(V64 dst, const std::vector<const CpuNTTPlan*>& ntt, DataDim dim) const {
        ntt_dim_impl(dst, ntt, dim, false, true);
    }
    void hal_intt_mont64_dim(V64 dst, const std::vector<const CpuNTTPlan*>& ntt, DataDim dim) const {
        ntt_dim_impl(dst, ntt, dim, true, true);
    }
    void hal_ntt_mul_mont64_dim(V64 dst, const std::vector<const CpuNTTPlan*>& ntt, DataDim dim, V64 mul,
                                const std::vector<MontgomeryModulus>& mods) const {
        ntt_dim_impl(dst, ntt, dim, false, false);
        hal_mul_mont64(dst, mul, mods);
    }
    /// default methods of the trait (src/hal/mod.rs:241-250)
    void hal_ntt_mont64(V64 dst, const std::vector<const CpuNTTPlan*>& dim2,
                        const std::vector<const CpuNTTPlan*>& dim3) const {
        hal_ntt_mont64_dim(dst, dim2, DataDim::Dim2);
        hal_ntt_mont64_dim(dst, dim3, DataDim::Dim3);
    }
    void hal_intt_mont64(V64 dst, const std::vector<const CpuNTTPlan*>& dim2,
                         const std::vector<const CpuNTTPlan*>& dim3) const {
        hal_intt_mont64_dim(dst, dim2, DataDim::Dim2);
        hal_intt_mont64_dim(dst, dim3, DataDim::Dim3);
    }

    // ---- base-conversion corrections (src/hal/cpu.rs:950-1057) ----
    void hal_bconv_correct_mont64(V64 dst, V128 lhs, V64 rhs, const std::vector<MontgomeryModulus>& mods,
                                  size_t shift) const {
        size_t i_len = dst.shape[0], j_len = dst.shape[1], k_len = dst.shape[2], l_len = dst.shape[3];
        ORACLE_ASSERT(shift >= 64 && shift < 127, "bconv_correct shift");
        ORACLE_ASSERT(lhs.shape == (Shape{i_len, 1, k_len, l_len}), "bconv_correct lhs shape");
        ORACLE_ASSERT(rhs.shape[0] == i_len || rhs.shape[0] == 1, "bconv_correct rhs dim 0");
        ORACLE_ASSERT(rhs.shape[1] == j_len && rhs.shape[2] == 1 && rhs.shape[3] == 1, "bconv_correct rhs shape");
        ORACLE_ASSERT(mods.size() == j_len, "moduli count");
        i128 half = (i128)1 << (shift - 1);
        for (size_t i = 0; i < i_len; i++) {
            size_t ri = rhs.shape[0] == 1 ? 0 : i;
            for (size_t j = 0; j < j_len; j++) {
                const MontgomeryModulus& m = mods[j];
                i128 r = (i128)rhs.at(ri, j, 0, 0);
                for (size_t k = 0; k < k_len; k++) {
                    int64_t* dl = dst.line(i, j, k);
                    const i128* ll = lhs.line(i, 0, k);
                    for (size_t l = 0; l < l_len; l++)
                        dl[l] = wadd(dl[l], m.red128(wmul128(wadd128(ll[l], half) >> shift, r)));
                }
            }
        }
    }
    void hal_bconv_correct_pow2(V64 dst, V128 src, int64_t factor0, int64_t factor1, size_t shift,
                                size_t log2_modulus) const {
        size_t i_len = dst.shape[0], k_len = dst.shape[2], l_len = dst.shape[3];
        ORACLE_ASSERT(dst.shape[1] == 1, "bconv_correct_pow2 dst shape");
        ORACLE_ASSERT(src.shape == (Shape{i_len, 2, k_len, l_len}), "bconv_correct_pow2 src shape");
        ORACLE_ASSERT(shift >= 1 && shift < 127, "shift");
        ORACLE_ASSERT(log2_modulus >= 1 && log2_modulus <= 62, "log2_modulus");
        i128 half = (i128)1 << (shift - 1);
        i128 modulus = (i128)1 << log2_modulus;
        i128 modulus_half = modulus / 2;
        for (size_t i = 0; i < i_len; i++)
            for (size_t k = 0; k < k_len; k++) {
                int64_t* dl = dst.line(i, 0, k);
                const i128* vl = src.line(i, 0, k);
                const i128* cl = src.line(i, 1, k);
                for (size_t l = 0; l < l_len; l++) {
                    i128 quot = wadd128(cl[l], half) >> shift;
                    i128 reduced =
                        rem_euclid128(wmul128(wsub128(vl[l], wmul128(quot, (i128)factor0)), (i128)factor1), modulus);
                    dl[l] = (int64_t)(reduced > modulus_half ? reduced - modulus : reduced);
                }
            }
    }
    void hal_bconv_correct_pow2_wide(V64 dst, V128 src, i128 factor0, i128 factor1, size_t shift,
                                     size_t log2_modulus) const {
        size_t i_len = dst.shape[0], k_len = dst.shape[2], l_len = dst.shape[3];
        ORACLE_ASSERT(dst.shape[1] == 2, "bconv_correct_pow2_wide dst shape");
        ORACLE_ASSERT(src.shape == (Shape{i_len, 3, k_len, l_len}), "bconv_correct_pow2_wide src shape");
        ORACLE_ASSERT(shift >= 1 && shift < 127, "shift");
        ORACLE_ASSERT(log2_modulus >= 1 && log2_modulus <= 126, "log2_modulus");
        i128 half = (i128)1 << (shift - 1);
        i128 modulus = (i128)1 << log2_modulus;
        i128 modulus_half = modulus / 2;
        for (size_t i = 0; i < i_len; i++)
            for (size_t k = 0; k < k_len; k++) {
                const i128* lo = src.line(i, 0, k);
                const i128* hi = src.line(i, 1, k);
                const i128* corr = src.line(i, 2, k);
                int64_t* d0 = dst.line(i, 0, k);
                int64_t* d1 = dst.line(i, 1, k);
                for (size_t l = 0; l < l_len; l++) {
                    i128 quot = wadd128(corr[l], half) >> shift;
                    i128 v = wadd128(lo[l], (i128)((u128)hi[l] << 64));
                    i128 reduced = rem_euclid128(wmul128(wsub128(v, wmul128(quot, factor0)), factor1), modulus);
                    i128 c = reduced > modulus_half ? reduced - modulus : reduced;
                    // split_i128_limbs (src/hal/mod.rs:71-76)
                    int64_t l0 = (int64_t)c;
                    int64_t h0 = (int64_t)((c - (i128)l0) >> 64);
                    d0[l] = l0;
                    d1[l] = h0;
                }
            }
    }

    // ---- permutations (src/hal/cpu.rs:1059-1122) ----
    CpuPermutationPlan hal_create_permutation(const std::vector<size_t>& inner_shape,
                                              const std::vector<size_t>& shifts) const {
        ORACLE_ASSERT(inner_shape.size() == shifts.size(), "permutation shape/shift length");
        size_t n = 1;
        for (size_t m : inner_shape) n *= m;
        CpuPermutationPlan plan;
        plan.len = n;
        std::vector<size_t> idx(inner_shape.size(), 0);
        for (size_t e = 0; e < n; e++) {
            size_t src = 0;
            for (size_t t = 0; t < inner_shape.size(); t++) {
                size_t m = inner_shape[t];
                src = src * m + (idx[t] + m - shifts[t] % m) % m;
            }
            plan.perm.push_back((uint32_t)src);
            for (size_t t = inner_shape.size(); t-- > 0;) {
                idx[t]++;
                if (idx[t] < inner_shape[t]) break;
                idx[t] = 0;
            }
        }
        return plan;
    }
    void hal_permute(V64 dst, V64 src, const CpuPermutationPlan& plan, DataDim dim) const {
        ORACLE_ASSERT(dst.shape == src.shape, "permute shapes");
        if (dim == DataDim::Dim2) {
            ORACLE_ASSERT(plan.len == dst.shape[2], "permutation length (dim 2)");
            for (size_t i = 0; i < dst.shape[0]; i++)
                for (size_t j = 0; j < dst.shape[1]; j++)
                    for (size_t e = 0; e < dst.shape[2]; e++)
                        std::memcpy(dst.line(i, j, e), src.line(i, j, plan.perm[e]), dst.shape[3] * sizeof(int64_t));
        } else {
            ORACLE_ASSERT(plan.len == dst.shape[3], "permutation length (dim 3)");
            for (size_t i = 0; i < dst.shape[0]; i++)
                for (size_t j = 0; j < dst.shape[1]; j++)
                    for (size_t k = 0; k < dst.shape[2]; k++) {
                        int64_t* dl = dst.line(i, j, k);
                        const int64_t* sl = src.line(i, j, k);
                        for (size_t l = 0; l < dst.shape[3]; l++) dl[l] = sl[plan.perm[l]];
                    }
        }
    }
};

}  // namespace oracle

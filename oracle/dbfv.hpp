// Oracle (test infrastructure only): CPU restatement of the dBFV pieces of the homomorphic CRT
// transform's baby-step / giant-step step, over the restated hal::cpu backend:
//   DBFVModulus, balanced_digits_vec             cyclosubfield-dbfv/src/dbfv.rs:56-121
//   DBFVAccumulator, allocate / add               src/dbfv.rs:124-163
//   fma / inner product with L' elements          src/dbfv.rs:193-260, 291-399
//   finish_accumulator, hom_fma_element_lprime    src/dbfv.rs:401-453
//   bsgs_split, pow_mod_m, galois elements        src/bootstrap/homcrt.rs:322-367
//   hom_cyclic_transform_dbfv                     src/bootstrap/homcrt.rs:369-429
#pragma once
#include "bfv.hpp"

namespace oracle {

/// src/dbfv.rs:56-81: t = 2^log2_t with digit base b = 2^log2_b
struct DBFVModulus {
    size_t log2_b, log2_t;
    size_t digits() const { return (log2_t - 1) / log2_b + 1; }
    i128 b() const { return (i128)1 << log2_b; }
};

/// src/dbfv.rs:97-121
inline std::vector<std::vector<i128>> balanced_digits_vec(const std::vector<i128>& x, i128 b, size_t max_digits) {
    std::vector<std::vector<i128>> result;
    std::vector<i128> current = x;
    for (size_t it = 0; it < max_digits; it++) {
        bool all_zero = true;
        for (i128 v : current) all_zero = all_zero && v == 0;
        if (all_zero) break;
        std::vector<i128> rems;
        for (i128& v : current) {
            i128 rem = cmod(v, b);
            rems.push_back(rem);
            v = (v - rem) / b;
        }
        result.push_back(rems);
    }
    return result;
}

/// src/dbfv.rs:124-150
struct DBFVAccumulator {
    WideRingEls acc;
    DBFVModulus modulus;
    Basis basis;
    size_t used_digits = 0;
    size_t capacity() const { return modulus.digits(); }
};

struct Dbfv {
    RingContext& ring;

    size_t digit_count(const RingView& ct) const {
        ORACLE_ASSERT(ct.count() % 2 == 0, "dBFV ciphertext rows");
        return ct.count() / 2;
    }
    DBFVAccumulator allocate_accumulator(DBFVModulus m, const Base& base, Basis basis) {
        return DBFVAccumulator{ring.allocate_wide(2 * m.digits(), base), m, basis, 0};
    }
    /// src/dbfv.rs:153-163
    void acc_add(DBFVAccumulator& acc, const RingView& ct) {
        size_t d = digit_count(ct);
        if (d == 0) return;
        ORACLE_ASSERT(d <= acc.capacity() && acc.basis == ct.basis && acc.acc.rns_base == ct.rns_base, "acc_add");
        acc.acc.add(ring.backend, 0, 2 * d, ct.data, ct.bound);
        acc.used_digits = std::max(acc.used_digits, d);
    }
    std::vector<Tensor<int64_t>> lprime_digit_tensors(const DBFVAccumulator& acc, const std::vector<i128>& rhs) {
        std::vector<Tensor<int64_t>> out;
        for (auto& coeffs : balanced_digits_vec(rhs, acc.modulus.b(), acc.modulus.digits()))
            out.push_back(ring.lprime_element_tensor(acc.acc.rns_base, coeffs));
        return out;
    }
    /// src/dbfv.rs:193-224
    void acc_fma_tensors(DBFVAccumulator& acc, const RingView& lhs, const std::vector<Tensor<int64_t>>& rhs) {
        size_t ld = digit_count(lhs);
        if (ld == 0 || rhs.empty()) return;
        ORACLE_ASSERT(ld <= acc.capacity() && acc.basis == lhs.basis && acc.acc.rns_base == lhs.rns_base, "acc_fma");
        size_t new_digits = std::min(acc.capacity(), ld + rhs.size() - 1);
        for (size_t i = 0; i < ld; i++)
            for (size_t j = 0; j < rhs.size(); j++) {
                size_t k = i + j;
                if (k < new_digits)
                    acc.acc.fma(ring.backend, 2 * k, 2 * k + 2, lhs.data.rows(2 * i, 2 * i + 2), lhs.bound,
                                rhs[j].view(), 1);
            }
        acc.used_digits = std::max(acc.used_digits, new_digits);
    }
    /// src/dbfv.rs:291-352
    void acc_inner_product_tensors(DBFVAccumulator& acc,
                                   const std::vector<std::pair<RingView, std::vector<Tensor<int64_t>>>>& terms) {
        size_t cap = acc.capacity(), max_new = 0;
        for (auto& t : terms) {
            size_t ld = digit_count(t.first);
            if (ld == 0 || t.second.empty()) continue;
            ORACLE_ASSERT(ld <= cap && acc.basis == t.first.basis && acc.acc.rns_base == t.first.rns_base,
                          "acc_inner_product");
            max_new = std::max(max_new, std::min(cap, ld + t.second.size() - 1));
        }
        if (max_new == 0) return;
        for (size_t k = 0; k < max_new; k++) {
            std::vector<std::tuple<V64, u128, V64, u128>> kt;
            for (auto& t : terms) {
                size_t ld = digit_count(t.first);
                if (ld == 0 || t.second.empty()) continue;
                size_t new_digits = std::min(cap, ld + t.second.size() - 1);
                if (k >= new_digits) continue;
                for (size_t j = 0; j < t.second.size(); j++) {
                    if (k < j) break;
                    size_t i = k - j;
                    if (i >= ld) continue;
                    kt.emplace_back(t.first.data.rows(2 * i, 2 * i + 2), t.first.bound, t.second[j].view(), 1);
                }
            }
            if (!kt.empty()) acc.acc.inner_product(ring.backend, 2 * k, 2 * k + 2, kt);
        }
        acc.used_digits = std::max(acc.used_digits, max_new);
    }
    /// src/dbfv.rs:401-404
    RingEls finish(const DBFVAccumulator& acc) { return ring.reduce_wide_rows(acc.acc, 0, 2 * acc.used_digits, acc.basis); }
    RingEls empty(const Base& base, Basis basis) { return ring.allocate_in_basis(0, base, basis); }
    /// src/dbfv.rs:431-453
    RingEls hom_fma_element_lprime(DBFVModulus m, const RingView& lhs, const std::vector<i128>& rhs,
                                   const RingView& summand) {
        ORACLE_ASSERT(lhs.basis == Basis::CRTBasis && summand.basis == Basis::CRTBasis, "CRT basis required");
        bool all_zero = true;
        for (i128 v : rhs) all_zero = all_zero && v == 0;
        if (digit_count(lhs) == 0 || all_zero) return ring.clone_els(summand);
        DBFVAccumulator acc = allocate_accumulator(m, lhs.rns_base, Basis::CRTBasis);
        acc_add(acc, summand);
        acc_fma_tensors(acc, lhs, lprime_digit_tensors(acc, rhs));
        return finish(acc);
    }
};

/// src/bootstrap/homcrt.rs:335-339
inline std::pair<size_t, size_t> bsgs_split(size_t len) {
    const size_t UNHOISTED_OVERHEAD = 3;  // homcrt.rs:333
    size_t best = 1, best_cost = (size_t)-1;
    for (size_t count = 1; count <= len; count++) {
        size_t cost = count + UNHOISTED_OVERHEAD * ((len - 1) / count + 1);
        if (cost < best_cost) best_cost = cost, best = count;
    }
    return {best, (len - 1) / best + 1};
}

/// src/bootstrap/homcrt.rs:341-347
inline uint64_t pow_mod_m(uint64_t g, size_t e, uint64_t m) {
    uint64_t r = 1;
    for (size_t i = 0; i < e; i++) r = (uint64_t)((u128)r * g % m);
    return r;
}

/// The Galois elements one cyclic transform of length `len` by `g` needs (homcrt.rs:350-361).
inline std::vector<uint64_t> transform_galois_elements(uint64_t g, size_t len, uint64_t m) {
    std::vector<uint64_t> out;
    if (len <= 1) return out;
    auto sp = bsgs_split(len);
    for (size_t j = 1; j < sp.first; j++) out.push_back(pow_mod_m(g, j, m));
    if (sp.second > 1) out.push_back(pow_mod_m(g, sp.first, m));
    return out;
}

/// src/bootstrap/homcrt.rs:369-429: Σ_i coeffs[i] σ^i(ct) with baby steps sharing the gadget
/// decomposition and giant steps applying one unhoisted automorphism to the accumulated result.
/// `key_for(g)` returns the Galois key of automorphism g.
inline RingEls hom_cyclic_transform_dbfv(RingContext& ring, DBFVModulus modulus, uint64_t automorphism,
                                         const std::vector<std::vector<i128>>& coeffs, const RingView& ct,
                                         const std::function<const KeySwitchKey*(uint64_t)>& key_for) {
    Dbfv D{ring};
    uint64_t st = 0;
    Bfv bfv(ring, &st);
    const size_t len = coeffs.size();
    const Base base = ct.rns_base;
    if (len == 0) return D.empty(base, Basis::CRTBasis);
    if (len == 1) {
        RingEls summand = D.empty(base, Basis::CRTBasis);
        return D.hom_fma_element_lprime(modulus, ct, coeffs[0], as_view(summand));
    }
    auto sp = bsgs_split(len);
    const size_t baby_steps = sp.first, giant_steps = sp.second;
    const uint64_t m = ring.field.m;
    const size_t d = D.digit_count(ct);
    std::vector<uint64_t> baby_exps;
    std::vector<const KeySwitchKey*> baby_keys;
    for (size_t j = 1; j < baby_steps; j++) {
        baby_exps.push_back(pow_mod_m(automorphism, j, m));
        baby_keys.push_back(key_for(baby_exps.back()));
    }
    std::vector<RingEls> babys;
    babys.push_back(ring.clone_els(ct));
    for (size_t j = 1; j < baby_steps; j++) babys.push_back(ring.allocate_in_basis(2 * d, base, Basis::CRTBasis));
    for (size_t di = 0; di < d; di++) {
        std::vector<RingEls> rot = bfv.bfv_hom_gal(as_view(babys[0]).rows(2 * di, 2 * di + 2), baby_exps, baby_keys);
        for (size_t j = 0; j < rot.size(); j++)
            ring.backend.hal_assign(babys[j + 1].data.view().rows(2 * di, 2 * di + 2), rot[j].data.view());
    }
    const uint64_t giant_exp = pow_mod_m(automorphism, baby_steps, m);
    RingEls out = D.empty(base, Basis::CRTBasis);
    for (size_t giant = giant_steps; giant-- > 0;) {
        if (giant != giant_steps - 1) {
            size_t od = D.digit_count(as_view(out));
            RingEls rotated = ring.allocate_in_basis(2 * od, base, Basis::CRTBasis);
            for (size_t di = 0; di < od; di++) {
                std::vector<RingEls> r =
                    bfv.bfv_hom_gal(as_view(out).rows(2 * di, 2 * di + 2), {giant_exp}, {key_for(giant_exp)});
                ring.backend.hal_assign(rotated.data.view().rows(2 * di, 2 * di + 2), r[0].data.view());
            }
            out = std::move(rotated);
        }
        DBFVAccumulator acc = D.allocate_accumulator(modulus, base, Basis::CRTBasis);
        std::vector<std::pair<RingView, std::vector<Tensor<int64_t>>>> terms;
        size_t nt = std::min(baby_steps, len - giant * baby_steps);
        for (size_t j = 0; j < nt; j++)
            terms.emplace_back(as_view(babys[j]), D.lprime_digit_tensors(acc, coeffs[giant * baby_steps + j]));
        D.acc_inner_product_tensors(acc, terms);
        D.acc_add(acc, as_view(out));
        out = D.finish(acc);
    }
    return out;
}

}  // namespace oracle

// ORACLE — test infrastructure only (see arith.hpp). Restates the hard-coded field descriptors
// and the group bookkeeping of cyclosubfield-dbfv/src/field.rs:
//   subgroup_elements          src/field.rs:52-67
//   FieldDescriptor::new       src/field.rs:157-215
//   transversals               src/field.rs:299-331
//   gal_to_shift, coset_index  src/field.rs:338-352
//   rou_order                  src/field.rs:440
//   inv_mod, crt2              src/field.rs:498-520
//   field_2/18/192/36864/49152 src/field.rs:529-540, 634-645, 675-686, 718-729, 758-769
// The per-prime bootstrapping data (src/field.rs:217-253) is not needed on the HAL path.
#pragma once
#include <algorithm>
#include <map>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include "arith.hpp"

namespace oracle {

inline uint64_t fmul_mod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128)a * b) % m); }

/// src/field.rs:52-67
inline std::vector<uint64_t> subgroup_elements(const std::vector<uint64_t>& gens, uint64_t m) {
    std::set<uint64_t> elements{1};
    std::vector<uint64_t> frontier{1};
    while (!frontier.empty()) {
        uint64_t x = frontier.back();
        frontier.pop_back();
        for (uint64_t g : gens) {
            uint64_t y = fmul_mod(x, g, m);
            if (elements.insert(y).second) frontier.push_back(y);
        }
    }
    return std::vector<uint64_t>(elements.begin(), elements.end());
}

inline uint64_t gcd_u64(uint64_t a, uint64_t b) { return b == 0 ? a : gcd_u64(b, a % b); }
inline uint64_t lcm_u64(uint64_t a, uint64_t b) { return a / gcd_u64(a, b) * b; }

/// src/field.rs:498-508
inline uint64_t inv_mod(uint64_t a, uint64_t n) {
    i128 old_r = (i128)a % (i128)n, r = (i128)n;
    i128 old_s = 1, s = 0;
    while (r != 0) {
        i128 q = old_r / r;
        i128 tmp = r;
        r = old_r - q * r;
        old_r = tmp;
        tmp = s;
        s = old_s - q * s;
        old_s = tmp;
    }
    ORACLE_ASSERT(old_r == 1 || old_r == -1, "elements are not coprime");
    return (uint64_t)rem_euclid128(old_s * old_r, (i128)n);
}

/// src/field.rs:511-520
inline uint64_t crt2(uint64_t a1, uint64_t m1, uint64_t a2, uint64_t m2) {
    if (m1 == 1) return a2 % m2;
    if (m2 == 1) return a1 % m1;
    uint64_t m1_inv_mod_m2 = inv_mod(m1 % m2, m2);
    uint64_t k = fmul_mod((a2 + m2 - a1 % m2) % m2, m1_inv_mod_m2, m2);
    return (uint64_t)(((u128)a1 + (u128)m1 * k) % ((u128)m1 * m2));
}

struct FieldDescriptorData {
    uint64_t m;
    uint64_t m_prime;
    std::vector<uint64_t> gal_mprime_lprime_gens;
    std::vector<uint64_t> gal_mk_k_gens;
    std::vector<std::pair<uint64_t, size_t>> gal_lprime_q_cyclic;
    std::vector<std::pair<uint64_t, size_t>> gal_kq_cyclic;
};

struct FieldDescriptor {
    std::string name;
    uint64_t m, m_prime;
    std::vector<uint64_t> m_factors;
    std::vector<std::pair<uint64_t, size_t>> lq_cyclic;
    size_t lprime_factor_count;
    size_t deg_l, deg_k, deg_lprime;
    std::vector<uint64_t> gal_ml, gal_mprime_lprime, gal_mk_k;
    std::map<uint64_t, size_t> transversal_index;

    /// src/field.rs:157-215
    static FieldDescriptor create(const std::string& name, const FieldDescriptorData& data) {
        FieldDescriptor f;
        f.name = name;
        f.m = data.m;
        f.m_prime = data.m_prime;
        ORACLE_ASSERT(f.m % 2 == 1, "m must be odd");
        if (data.m_prime != 1) f.m_factors.push_back(data.m_prime);
        uint64_t rest = f.m / data.m_prime;
        for (uint64_t p = 3; rest > 1; p += 2)
            if (rest % p == 0) {
                rest /= p;
                ORACLE_ASSERT(rest % p != 0, "m must be squarefree");
                f.m_factors.push_back(p);
            }
        uint64_t phi_m = 1;
        for (uint64_t p : f.m_factors) phi_m *= p - 1;
        f.gal_mprime_lprime = subgroup_elements(data.gal_mprime_lprime_gens, f.m);
        f.gal_mk_k = subgroup_elements(data.gal_mk_k_gens, f.m);
        std::vector<uint64_t> all_gens = data.gal_mprime_lprime_gens;
        all_gens.insert(all_gens.end(), data.gal_mk_k_gens.begin(), data.gal_mk_k_gens.end());
        f.gal_ml = subgroup_elements(all_gens, f.m);
        f.lq_cyclic = data.gal_lprime_q_cyclic;
        f.lq_cyclic.insert(f.lq_cyclic.end(), data.gal_kq_cyclic.begin(), data.gal_kq_cyclic.end());
        f.lprime_factor_count = data.gal_lprime_q_cyclic.size();
        f.deg_l = 1;
        for (auto& c : f.lq_cyclic) f.deg_l *= c.second;
        f.deg_lprime = 1;
        for (auto& c : data.gal_lprime_q_cyclic) f.deg_lprime *= c.second;
        f.deg_k = f.deg_l / f.deg_lprime;
        ORACLE_ASSERT(phi_m == f.deg_l * f.gal_ml.size(), "transversal size must match [L : Q]");
        std::vector<uint64_t> tr = f.lq_transversal();
        for (size_t i = 0; i < tr.size(); i++) {
            bool fresh = f.transversal_index.emplace(tr[i], i).second;
            ORACLE_ASSERT(fresh, "generators do not induce an isomorphism");
        }
        return f;
    }

    uint64_t m_k() const { return m / m_prime; }

    /// src/field.rs:299-317
    std::vector<uint64_t> transversal_of(const std::vector<std::pair<uint64_t, size_t>>& factors) const {
        std::vector<uint64_t> result{1};
        for (auto& [g, n] : factors) {
            std::vector<uint64_t> powers;
            uint64_t power = 1;
            for (size_t i = 0; i < n; i++) {
                powers.push_back(power);
                power = fmul_mod(power, g, m);
            }
            std::vector<uint64_t> next;
            for (uint64_t x : result)
                for (uint64_t p : powers) next.push_back(fmul_mod(x, p, m));
            result = next;
        }
        return result;
    }
    std::vector<std::pair<uint64_t, size_t>> lprime_q_cyclic() const {
        return std::vector<std::pair<uint64_t, size_t>>(lq_cyclic.begin(), lq_cyclic.begin() + lprime_factor_count);
    }
    std::vector<std::pair<uint64_t, size_t>> kq_cyclic() const {
        return std::vector<std::pair<uint64_t, size_t>>(lq_cyclic.begin() + lprime_factor_count, lq_cyclic.end());
    }
    std::vector<uint64_t> lq_transversal() const { return transversal_of(lq_cyclic); }
    std::vector<uint64_t> kq_transversal() const { return transversal_of(kq_cyclic()); }
    std::vector<uint64_t> lprime_q_transversal() const { return transversal_of(lprime_q_cyclic()); }
    std::vector<size_t> lq_cyclic_orders() const {
        std::vector<size_t> r;
        for (auto& c : lq_cyclic) r.push_back(c.second);
        return r;
    }
    std::vector<size_t> lprime_orders() const {
        std::vector<size_t> r;
        for (size_t i = 0; i < lprime_factor_count; i++) r.push_back(lq_cyclic[i].second);
        return r;
    }
    std::vector<size_t> k_orders() const {
        std::vector<size_t> r;
        for (size_t i = lprime_factor_count; i < lq_cyclic.size(); i++) r.push_back(lq_cyclic[i].second);
        return r;
    }

    /// src/field.rs:349-352
    bool coset_index(uint64_t g, size_t* out) const {
        ORACLE_ASSERT(gcd_u64(g % m, m) == 1, "not an element of (Z/mZ)*");
        for (uint64_t h : gal_ml) {
            auto it = transversal_index.find(fmul_mod(g % m, h, m));
            if (it != transversal_index.end()) {
                *out = it->second;
                return true;
            }
        }
        return false;
    }

    /// src/field.rs:338-346
    std::vector<int64_t> gal_to_shift(uint64_t g) const {
        size_t index;
        ORACLE_ASSERT(coset_index(g, &index), "inconsistent subgroup data");
        std::vector<int64_t> result(lq_cyclic.size(), 0);
        for (size_t i = lq_cyclic.size(); i-- > 0;) {
            result[i] = (int64_t)(index % lq_cyclic[i].second);
            index /= lq_cyclic[i].second;
        }
        return result;
    }

    /// src/field.rs:440
    uint64_t rou_order() const {
        uint64_t l = 1;
        for (auto& c : lq_cyclic) l = lcm_u64(l, c.second);
        return m * l;
    }

    /// src/field.rs:447
    int64_t scale_q_to_m_period_basis() const { return m_factors.size() % 2 == 1 ? -1 : 1; }
};

/// The hard-coded descriptors, by name (src/field.rs:529-769).
inline FieldDescriptor field_by_name(const std::string& name) {
    if (name == "field_36864")
        return FieldDescriptor::create(
            name, {8536255, 13, {}, {3283177}, {{3939811, 4}, {7879621, 3}},
                   {{7316791, 2}, {1169351, 3}, {4560466, 8}, {8071246, 64}}});
    if (name == "field_49152")
        return FieldDescriptor::create(
            name, {35297665, 13, {29867256}, {2715207}, {{32582461, 4}}, {{1291681, 3}, {20965738, 64}, {30783429, 64}}});
    if (name == "field_192")
        return FieldDescriptor::create(name,
                                       {90627, 3, {}, {30211}, {{60419, 2}}, {{45427, 2}, {4183, 3}, {47533, 16}}});
    if (name == "field_18")
        return FieldDescriptor::create(name, {1729, 19, {274}, {457}, {{1548, 3}}, {{1483, 2}, {932, 3}}});
    if (name == "field_16") return FieldDescriptor::create(name, {257, 1, {}, {2}, {}, {{155, 16}}});
    if (name == "field_2") return FieldDescriptor::create(name, {7, 1, {}, {2}, {}, {{6, 2}}});
    if (name == "field_32") return FieldDescriptor::create(name, {255, 17, {}, {137}, {{241, 16}}, {{52, 2}}});
    fail("unknown field " + name);
}

}  // namespace oracle

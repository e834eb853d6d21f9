// Ring and BFV layers on the GPU (include/ringcuda.h).
//
// Host-side state mirrors the reference's RingContext (cyclosubfield-dbfv/src/ring.rs:594-652):
// the field's group data, the RNS factors with their Montgomery moduli and NTT plans, the
// NTT-domain CRT kernels, and caches for base conversions, gadget conversions and Galois
// permutations. All constants are computed on the host without big integers (products of primes
// are evaluated modulo each prime). The per-element work runs as sm_103a kernels: the HAL kernels
// for transforms and pointwise steps, and the fused kernels of ring_kernels.cu for base
// conversion, key switching, Galois automorphisms and tensor products.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <set>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/ringcuda.h"
#include "common.cuh"

namespace hc {
hc_status launch_bconv_fused(hc_context ctx, const KView& src, const KView& dst, const BconvConsts& c, int r, int rd,
                             int nb, const KMods& sm, const KMods& dm, int64_t ns, const int64_t* sub_mul);
hc_status launch_galois(hc_context ctx, const KView& d, const KView& s, const uint32_t* p2, const uint32_t* p3);
hc_status launch_keyswitch(hc_context ctx, const KView* parts, const KView* keys, int nterms, const KView* add0,
                           const KView* add1, int full0, int full1, const KView& dst, const KMods& m,
                           const int64_t* one_dev, const uint32_t* p2, const uint32_t* p3, bool reverse = false);
hc_status launch_tensor(hc_context ctx, const KView& d, const KView& lhs_lo, const KView& lhs_hi, const KView& rhs_lo,
                        const KView& rhs_hi, int rsplit, const KMods& m, int f0,
                        int f1, int f2);
bool crt_pass_ready(hc_context ctx, const hc_ntt_plan* plans2, const hc_ntt_plan* plans3, size_t r, const KView& t);
hc_status launch_crt_pass(hc_context ctx, int dir, const KView& t, const KView* src, const hc_ntt_plan* plans2,
                          const hc_ntt_plan* plans3, size_t r, const KView& m2, const KView& m3, bool post,
                          const KMods& mods);
hc_status launch_giant(hc_context ctx, const KView& babies, const KView& lcoef, int nbaby, int d, const int* lfirst,
                       const int* lcount, const KView* add, int nadd, const unsigned char* full, int used,
                       const KView& dst, const KMods& m, const int64_t* one_dev);
size_t crt_slab_tile_words(int32_t shapes, int32_t dl, int32_t dk, int logv);
}  // namespace hc

using namespace hc;

namespace {

const i128 I128MAX = (i128)(~(u128)0 >> 1);

struct Fail {
    hc_status st;
};
#define CK(expr)                                \
    do {                                        \
        hc_status _st = (expr);                 \
        if (_st != HC_OK) throw Fail{_st};      \
    } while (0)
#define REQUIRE(cond, st, msg)                  \
    do {                                        \
        if (!(cond)) throw Fail{fail(st, msg)}; \
    } while (0)

template <typename F>
hc_status guard(F f) {
    try {
        f();
        return HC_OK;
    } catch (const Fail& e) {
        return e.st;
    } catch (const std::exception& e) {
        return fail(HC_ERR_ARG, e.what());
    }
}

// ------------------------------------------------------------------------- integer helpers
int64_t mulm(int64_t a, int64_t b, int64_t p) { return (int64_t)(((i128)a * b) % p); }
int64_t emod(int64_t a, int64_t p) {
    int64_t r = a % p;
    return r < 0 ? r + p : r;
}
int64_t powm(int64_t b, uint64_t e, int64_t p) {
    int64_t r = 1;
    b = emod(b, p);
    while (e) {
        if (e & 1) r = mulm(r, b, p);
        b = mulm(b, b, p);
        e >>= 1;
    }
    return r;
}
int64_t invm(int64_t a, int64_t p) { return powm(emod(a, p), (uint64_t)(p - 2), p); }
/// x * 2^64 mod p with the sign of x (Rust's truncating `%`, src/ring.rs:109)
int64_t mont_repr(int64_t x, int64_t p) { return (int64_t)(((i128)x << 64) % (i128)p); }
/// representative in [-(p-1)/2, (p-1)/2] (feanor-math smallest_lift)
int64_t centred(int64_t x, int64_t p) {
    x = emod(x, p);
    return x > (p - 1) / 2 ? x - p : x;
}
int64_t from_mont(int64_t x, int64_t p) { return mulm(emod(x, p), invm(mont_repr(1, p), p), p); }
uint64_t umulm(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

bool is_prime64(uint64_t n) {
    if (n < 2) return false;
    static const uint64_t bases[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t p : bases)
        if (n % p == 0) return n == p;
    uint64_t d = n - 1;
    int s = 0;
    while (!(d & 1)) d >>= 1, s++;
    for (uint64_t a : bases) {
        uint64_t x = 1, b = a % n, e = d;
        while (e) {
            if (e & 1) x = umulm(x, b, n);
            b = umulm(b, b, n);
            e >>= 1;
        }
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int i = 1; i < s && comp; i++) {
            x = umulm(x, x, n);
            if (x == n - 1) comp = false;
        }
        if (comp) return false;
    }
    return true;
}

size_t bitlen_u128(u128 v) {
    size_t b = 0;
    while (v) b++, v >>= 1;
    return b;
}

/// Exact bit length of a product of primes.
size_t product_bits(const std::vector<int64_t>& ps) {
    std::vector<uint64_t> limbs{1};
    for (int64_t p : ps) {
        u128 carry = 0;
        for (auto& w : limbs) {
            u128 t = (u128)w * (uint64_t)p + carry;
            w = (uint64_t)t;
            carry = t >> 64;
        }
        if (carry) limbs.push_back((uint64_t)carry);
    }
    return 64 * (limbs.size() - 1) + bitlen_u128(limbs.back());
}

// ------------------------------------------------------------------------- fields
/// Hard-coded field data (cyclosubfield-dbfv/src/field.rs:529-769): conductor m, the prime m',
/// generators of Gal(M'|L') and Gal(M_K|K) in (Z/mZ)*, and the cyclic decompositions
/// (generator, order) of Gal(L'|Q) and Gal(K|Q), L'-factors first.
struct FieldSpec {
    const char* name;
    uint64_t m, m_prime;
    std::vector<uint64_t> gens_lp, gens_k;
    std::vector<std::pair<uint64_t, size_t>> cyc_lp, cyc_k;
};

const std::vector<FieldSpec>& field_specs() {
    static const std::vector<FieldSpec> specs = {
        {"field_36864", 8536255, 13, {}, {3283177}, {{3939811, 4}, {7879621, 3}},
         {{7316791, 2}, {1169351, 3}, {4560466, 8}, {8071246, 64}}},
        {"field_49152", 35297665, 13, {29867256}, {2715207}, {{32582461, 4}},
         {{1291681, 3}, {20965738, 64}, {30783429, 64}}},
        {"field_192", 90627, 3, {}, {30211}, {{60419, 2}}, {{45427, 2}, {4183, 3}, {47533, 16}}},
        {"field_18", 1729, 19, {274}, {457}, {{1548, 3}}, {{1483, 2}, {932, 3}}},
        {"field_16", 257, 1, {}, {2}, {}, {{155, 16}}},
        {"field_2", 7, 1, {}, {2}, {}, {{6, 2}}},
        {"field_32", 255, 17, {}, {137}, {{241, 16}}, {{52, 2}}},
    };
    return specs;
}

struct Field {
    FieldSpec spec;
    std::vector<uint64_t> m_factors;
    std::vector<std::pair<uint64_t, size_t>> cyc;  // L' factors then K factors
    size_t nlp;                                    // number of L' factors
    size_t deg_l, deg_lp, deg_k;
    std::vector<uint64_t> gal_ml, gal_lp, gal_k;   // Gal(M|L), Gal(M'|L'), Gal(M_K|K)
    std::unordered_map<uint64_t, size_t> tindex;   // transversal element -> flat index

    uint64_t m() const { return spec.m; }
    uint64_t m_k() const { return spec.m / spec.m_prime; }

    static std::vector<uint64_t> subgroup(const std::vector<uint64_t>& gens, uint64_t m) {
        std::set<uint64_t> el{1};
        std::vector<uint64_t> todo{1};
        while (!todo.empty()) {
            uint64_t x = todo.back();
            todo.pop_back();
            for (uint64_t g : gens) {
                uint64_t y = umulm(x, g, m);
                if (el.insert(y).second) todo.push_back(y);
            }
        }
        return std::vector<uint64_t>(el.begin(), el.end());
    }
    /// elements g_1^e_1 ... g_k^e_k in row-major order of (e_1, ..., e_k)
    std::vector<uint64_t> transversal(size_t from, size_t to) const {
        std::vector<uint64_t> out{1};
        for (size_t f = from; f < to; f++) {
            std::vector<uint64_t> next;
            next.reserve(out.size() * cyc[f].second);
            for (uint64_t x : out) {
                uint64_t pw = 1;
                for (size_t e = 0; e < cyc[f].second; e++) {
                    next.push_back(umulm(x, pw, spec.m));
                    pw = umulm(pw, cyc[f].first, spec.m);
                }
            }
            out.swap(next);
        }
        return out;
    }
    std::vector<size_t> orders(size_t from, size_t to) const {
        std::vector<size_t> o;
        for (size_t f = from; f < to; f++) o.push_back(cyc[f].second);
        return o;
    }
    uint64_t rou_order() const {
        uint64_t l = 1;
        for (auto& c : cyc) {
            uint64_t a = l, b = c.second;
            while (b) std::swap(a, b), b %= a;
            l = l / a * c.second;
        }
        return spec.m * l;
    }
    /// exponents of g in the cyclic decomposition of Gal(L|Q) (src/field.rs:338-352)
    std::vector<size_t> gal_to_shift(uint64_t g) const {
        uint64_t gm = g % spec.m;
        size_t idx = (size_t)-1;
        for (uint64_t h : gal_ml) {
            auto it = tindex.find(umulm(gm, h, spec.m));
            if (it != tindex.end()) {
                idx = it->second;
                break;
            }
        }
        REQUIRE(idx != (size_t)-1, HC_ERR_ARG, "not an element of (Z/mZ)* / inconsistent field data");
        std::vector<size_t> s(cyc.size());
        for (size_t f = cyc.size(); f-- > 0;) {
            s[f] = idx % cyc[f].second;
            idx /= cyc[f].second;
        }
        return s;
    }

    static Field make(const std::string& name) {
        const FieldSpec* sp = nullptr;
        for (auto& s : field_specs())
            if (name == s.name) sp = &s;
        REQUIRE(sp, HC_ERR_ARG, "unknown field " + name);
        Field f;
        f.spec = *sp;
        if (sp->m_prime != 1) f.m_factors.push_back(sp->m_prime);
        uint64_t rest = sp->m / sp->m_prime;
        for (uint64_t p = 3; rest > 1; p += 2)
            if (rest % p == 0) rest /= p, f.m_factors.push_back(p);
        f.cyc = sp->cyc_lp;
        f.cyc.insert(f.cyc.end(), sp->cyc_k.begin(), sp->cyc_k.end());
        f.nlp = sp->cyc_lp.size();
        f.deg_l = f.deg_lp = 1;
        for (size_t i = 0; i < f.cyc.size(); i++) {
            f.deg_l *= f.cyc[i].second;
            if (i < f.nlp) f.deg_lp *= f.cyc[i].second;
        }
        f.deg_k = f.deg_l / f.deg_lp;
        f.gal_lp = subgroup(sp->gens_lp, sp->m);
        f.gal_k = subgroup(sp->gens_k, sp->m);
        std::vector<uint64_t> all = sp->gens_lp;
        all.insert(all.end(), sp->gens_k.begin(), sp->gens_k.end());
        f.gal_ml = subgroup(all, sp->m);
        std::vector<uint64_t> tr = f.transversal(0, f.cyc.size());
        for (size_t i = 0; i < tr.size(); i++) f.tindex[tr[i]] = i;
        return f;
    }
};

uint64_t inv_mod_u(uint64_t a, uint64_t n) {
    i128 r0 = (i128)(a % n), r1 = n, s0 = 1, s1 = 0;
    while (r1) {
        i128 q = r0 / r1, t = r0 - q * r1;
        r0 = r1, r1 = t;
        t = s0 - q * s1;
        s0 = s1, s1 = t;
    }
    i128 v = (s0 * r0) % (i128)n;
    return (uint64_t)(v < 0 ? v + n : v);
}
uint64_t crt2(uint64_t a1, uint64_t m1, uint64_t a2, uint64_t m2) {
    if (m1 == 1) return a2 % m2;
    if (m2 == 1) return a1 % m1;
    uint64_t k = umulm((a2 + m2 - a1 % m2) % m2, inv_mod_u(m1 % m2, m2), m2);
    return (uint64_t)(((u128)a1 + (u128)m1 * k) % ((u128)m1 * m2));
}

// ------------------------------------------------------------------------- prime sampling
/// Largest prime <= bound that is 1 mod m, stepping down (src/ring.rs:136-146).
int64_t prime_below(int64_t bound, int64_t m) {
    int64_t c = bound - (bound - 1) % m;
    while (!is_prime64((uint64_t)c)) {
        c -= m;
        REQUIRE(c > 0, HC_ERR_ARG, "no suitable prime");
    }
    return c;
}
/// Adds primes of at most `each` bits until the product has `min_bits` (src/ring.rs:150-183).
std::vector<int64_t> sample_primes(std::vector<int64_t> have, size_t min_bits, size_t max_bits, size_t each,
                                   int64_t m) {
    const std::vector<int64_t> start = have;
    double bits = 0;
    for (int64_t p : have) bits += std::log2((double)p);
    int64_t ub = (int64_t)1 << each;
    while (bits < (double)min_bits) {
        double remaining = (double)min_bits - bits, allowed;
        if (remaining < (double)each) allowed = std::fmin((double)max_bits - bits, (double)each);
        else allowed = std::fmin(((double)max_bits - bits) / std::ceil(remaining / (double)each), (double)each);
        ub = std::min(ub, (int64_t)1 << (size_t)std::floor(allowed));
        int64_t p = prime_below(ub, m);
        ub = p - 1;
        while (std::find(start.begin(), start.end(), p) != start.end()) {
            p = prime_below(ub, m);
            ub = p - 1;
        }
        bits += std::log2((double)p);
        have.push_back(p);
    }
    return have;
}

// ------------------------------------------------------------------------- device buffers
struct DBuf {
    hc_context ctx = nullptr;
    void* p = nullptr;
    DBuf() {}
    DBuf(hc_context c, size_t bytes) : ctx(c) {
        count_alloc();
        CK(cuda_check(cudaMallocAsync(&p, bytes ? bytes : 16, stream_of(c)), "ring buffer allocation"));
    }
    DBuf(hc_context c, const void* host, size_t bytes) : DBuf(c, bytes) {
        CK(cuda_check(cudaMemcpyAsync(p, host, bytes, cudaMemcpyHostToDevice, stream_of(c)), "ring table upload"));
        CK(cuda_check(cudaStreamSynchronize(stream_of(c)), "ring table upload"));
    }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : ctx(o.ctx), p(o.p) { o.p = nullptr; }
    DBuf& operator=(DBuf&& o) noexcept {
        std::swap(ctx, o.ctx);
        std::swap(p, o.p);
        return *this;
    }
    ~DBuf() {
        if (p) cudaFreeAsync(p, stream_of(ctx));
    }
    template <typename T>
    T* as() const {
        return (T*)p;
    }
};

/// An owned contiguous device tensor [n0, n1, n2, n3] of i64 or i128 entries.
struct Tensor {
    DBuf buf;
    int64_t shape[4] = {0, 0, 0, 0};
    bool wide = false;
    Tensor() {}
    /// `zero`: zero-filled like the reference's allocate; internal temporaries that are fully
    /// overwritten before being read skip the fill (it would cost one more pass over HBM)
    Tensor(hc_context c, int64_t a, int64_t b, int64_t cc, int64_t d, bool w = false, bool zero = true) : wide(w) {
        shape[0] = a, shape[1] = b, shape[2] = cc, shape[3] = d;
        if (zero) {
            CK(w ? hc_allocate_i128(c, shape, &buf.p) : hc_allocate_i64(c, shape, &buf.p));
        } else {
            size_t bytes = (size_t)(a * b * cc * d) * (w ? 16 : 8);
            count_alloc();
            CK(cuda_check(cudaMallocAsync(&buf.p, bytes ? bytes : 16, stream_of(c)), "temporary allocation"));
        }
        buf.ctx = c;
    }
    hc_view view() const {
        hc_view v;
        v.ptr = buf.p;
        for (int d = 0; d < 4; d++) v.shape[d] = shape[d];
        v.strides[3] = 1, v.strides[2] = shape[3], v.strides[1] = shape[2] * shape[3];
        v.strides[0] = shape[1] * shape[2] * shape[3];
        return v;
    }
};

size_t esize_of(bool wide) { return wide ? 16 : 8; }
/// rows [s, e) of dimension 0
hc_view vrows(hc_view v, int64_t s, int64_t e, bool wide = false) {
    v.ptr = (char*)v.ptr + s * v.strides[0] * (int64_t)esize_of(wide);
    v.shape[0] = e - s;
    return v;
}
/// every `step`-th row starting at `s`, `count` rows
hc_view vstep(hc_view v, int64_t s, int64_t step, int64_t count) {
    v.ptr = (char*)v.ptr + s * v.strides[0] * 8;
    v.shape[0] = count;
    v.strides[0] *= step;
    return v;
}
Tensor temp(hc_context c, int64_t a, int64_t b, int64_t cc, int64_t d) { return Tensor(c, a, b, cc, d, false, false); }
/// RNS rows [s, e) of dimension 1
hc_view vbase(hc_view v, int64_t s, int64_t e, bool wide = false) {
    v.ptr = (char*)v.ptr + s * v.strides[1] * (int64_t)esize_of(wide);
    v.shape[1] = e - s;
    return v;
}
KView kv(const hc_view& v) {
    KView k;
    k.p = (char*)v.ptr;
    k.n0 = v.shape[0], k.n1 = v.shape[1], k.n2 = v.shape[2], k.n3 = v.shape[3];
    k.s0 = v.strides[0], k.s1 = v.strides[1], k.s2 = v.strides[2];
    k.b3 = 0;
    return k;
}
void check_view(const hc_view& v, int64_t n0, int64_t n1, int64_t n2, int64_t n3, const char* what) {
    REQUIRE(v.shape[0] == n0 && v.shape[1] == n1 && v.shape[2] == n2 && v.shape[3] == n3, HC_ERR_SHAPE,
            std::string(what) + ": unexpected shape");
    REQUIRE(n3 <= 1 || v.strides[3] == 1, HC_ERR_SHAPE, std::string(what) + ": dimension 3 must be contiguous");
    REQUIRE(v.ptr || n0 * n1 * n2 * n3 == 0, HC_ERR_ARG, std::string(what) + ": null data");
}

typedef std::vector<size_t> Base;
typedef std::vector<std::pair<size_t, size_t>> Digits;

enum class Basis { PB, CRT };

// ------------------------------------------------------------------------- caches
struct Factor {
    int64_t p;
    hc_modulus mod;
    bool transform;
    hc_ntt_plan plan_lp = nullptr, plan_k = nullptr;
    std::vector<int64_t> kl, kk, ikl, ikk;  // NTT-domain CRT kernels (Montgomery form)
    bool have_kernels = false;
};

struct TransformCache {
    Base base;
    std::vector<hc_modulus> mods;
    std::vector<hc_ntt_plan> plp, pk;
    Tensor kl, kk, ikl, ikk;
};

/// Host mirror of the device Montgomery product mul_mont (the same integers).
int64_t mul_mont_host(int64_t a, int64_t b, int64_t n, int64_t ninv) {
    const i128 p = (i128)a * b;
    const uint64_t lo = (uint64_t)p;
    const int64_t m = (int64_t)(lo * (uint64_t)ninv);
    const int64_t thi = (int64_t)(((i128)m * n) >> 64);
    return (int64_t)((uint64_t)(int64_t)(p >> 64) + (uint64_t)thi + (uint64_t)(lo != 0));
}

/// Device tables of one base conversion in blocks (nb blocks of rd outputs over the source columns
/// ucol[b]), as bconv_fused_kernel reads them (BconvConsts):
///  - qinv / mat / qmodp / ucol: the reference's factors (the conversion matrix [nb][rd + 1][r] with
///    the correction row last in each block);
///  - mat3: the matrix rows 0..rd-1 as 29-bit limbs (m mod 2^29, m >> 29, their sum), for the
///    kernel's exact int64 multiply-accumulate; it needs |m| < 2^56 and lifts |x| < 2^57, i.e.
///    source primes below 2^57 (the ring's RNS factor size rule; checked here all the same);
///  - qinvp, r2p: the Montgomery factors qinv[u] and R^2 mod p_j times -p^-1 mod 2^64, so that the
///    kernel's products with them skip one 64-bit multiplication (mul_mont_c);
///  - qtab: mul_mont(q, qmodp) for every correction q in [-qhalf, qhalf] (|q| is at most the
///    block's source count, because 2^shift exceeds 4 r max(p)); larger q would be computed;
///  - corr_limb: whether the correction row (round(2^shift / p_u)) is small enough for the limb
///    products too.
struct BconvTables {
    DBuf qinv, qinvp, mat, mat3, qmodp, qtab, r2p, ucol;
    BconvConsts c{};
};

void build_bconv_tables(hc_context ctx, BconvTables& t, const std::vector<int64_t>& qinv,
                        const std::vector<hc_modulus>& sm, const std::vector<int64_t>& mat,
                        const std::vector<int64_t>& qm, const std::vector<hc_modulus>& dm,
                        const std::vector<int32_t>& uc, int shift, int chunk) {
    const size_t r = sm.size(), rd = dm.size(), nb = uc.size() / 2;
    int64_t maxsrc = 0;
    for (auto& m : sm) maxsrc = std::max(maxsrc, m.n);
    REQUIRE(maxsrc < ((int64_t)1 << 57), HC_ERR_UNSUPPORTED, "base conversion: source prime above 2^57");
    size_t maxlen = 0;
    for (size_t b = 0; b < nb; b++) maxlen = std::max(maxlen, (size_t)(uc[2 * b + 1] - uc[2 * b]));
    std::vector<int32_t> m3(nb * rd * r * 4, 0);
    std::vector<int64_t> qinvp(r), r2p(rd), qtab;
    int64_t maxmq = 0;
    for (size_t b = 0; b < nb; b++) {
        for (size_t j = 0; j < rd; j++)
            for (size_t u = 0; u < r; u++) {
                const int64_t m = mat[(b * (rd + 1) + j) * r + u];
                REQUIRE(m < ((int64_t)1 << 56) && m > -((int64_t)1 << 56), HC_ERR_UNSUPPORTED,
                        "base conversion: matrix entry above 2^56");
                const size_t o = ((b * rd + j) * r + u) * 4;
                m3[o] = (int32_t)(m & ((1 << 29) - 1));
                m3[o + 1] = (int32_t)(m >> 29);
                m3[o + 2] = m3[o] + m3[o + 1];
            }
        for (size_t u = 0; u < r; u++) maxmq = std::max(maxmq, std::abs(mat[(b * (rd + 1) + rd) * r + u]));
    }
    for (size_t u = 0; u < r; u++) qinvp[u] = (int64_t)((uint64_t)qinv[u] * (uint64_t)sm[u].neg_inv_n);
    for (size_t j = 0; j < rd; j++) r2p[j] = (int64_t)((uint64_t)dm[j].r2_mod_n * (uint64_t)dm[j].neg_inv_n);
    const int qhalf = (int)maxlen;
    for (size_t b = 0; b < nb; b++)
        for (size_t j = 0; j < rd; j++)
            for (int q = -qhalf; q <= qhalf; q++)
                qtab.push_back(mul_mont_host(q, qm[b * rd + j], dm[j].n, dm[j].neg_inv_n));
    t.qinv = DBuf(ctx, qinv.data(), r * 8);
    t.qinvp = DBuf(ctx, qinvp.data(), r * 8);
    t.mat = DBuf(ctx, mat.data(), mat.size() * 8);
    t.mat3 = DBuf(ctx, m3.data(), m3.size() * 4);
    t.qmodp = DBuf(ctx, qm.data(), qm.size() * 8);
    t.qtab = DBuf(ctx, qtab.data(), qtab.size() * 8);
    t.r2p = DBuf(ctx, r2p.data(), rd * 8);
    t.ucol = DBuf(ctx, uc.data(), uc.size() * 4);
    BconvConsts& c = t.c;
    c.qinv = t.qinv.as<int64_t>(), c.qinvp = t.qinvp.as<int64_t>(), c.mat = t.mat.as<int64_t>();
    c.mat3 = t.mat3.as<int4>(), c.qmodp = t.qmodp.as<int64_t>(), c.qtab = t.qtab.as<int64_t>();
    c.r2p = t.r2p.as<int64_t>(), c.ucol = t.ucol.as<int32_t>();
    c.qhalf = qhalf, c.shift = shift, c.chunk = chunk;
    // the correction row's limb products x0 mq, x1 mq summed over a block stay below 2^63
    c.corr_limb = maxmq < ((int64_t)1 << 30) && (i128)maxmq * ((i128)1 << 29) * (i128)maxlen < ((i128)1 << 63);
}

struct BconvCache {
    Base src, dst;
    BconvTables t;
};

struct GadgetCache {
    Base base;
    Digits digits;
    BconvTables t;
};

struct PermCache {
    DBuf p2, p3;
};

}  // namespace

struct hc_ring_s {
    hc_context ctx;
    // a second stream for independent branches of one call (SideBranch), with its fork / join events
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    void create_side() {
        CK(cuda_check(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "ring side stream"));
        CK(cuda_check(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming), "ring branch event"));
        CK(cuda_check(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming), "ring branch event"));
    }
    Field field;
    std::vector<Factor> factors;
    size_t initial_len = 0;
    size_t t_bits = 0;
    std::vector<std::unique_ptr<TransformCache>> tcache;
    std::vector<std::unique_ptr<BconvCache>> bcache;
    std::vector<std::unique_ptr<GadgetCache>> gcache;
    std::map<std::vector<size_t>, std::unique_ptr<PermCache>> pcache;
    std::map<Base, std::unique_ptr<DBuf>> one_cache;
    std::map<std::pair<Base, i128>, std::unique_ptr<Tensor>> scalar_cache;
    std::map<std::pair<Base, Base>, std::unique_ptr<Tensor>> qinv_cache;
    std::map<std::pair<Base, Base>, std::unique_ptr<DBuf>> qinv_pair_cache;
    // dBFV reduction tables (dbfv_tables) by (log2 b, log2 t, base), type-erased: their type is
    // defined with the dBFV code below
    std::map<std::tuple<size_t, size_t, Base>, std::shared_ptr<void>> dbfv_cache;
    // pinned staging of per-call host uploads (upload_async) and the event of its last copy
    void* stage = nullptr;
    size_t stage_bytes = 0;
    cudaEvent_t stage_ev = nullptr;

    /// Copies n host words into the contiguous device buffer dst on the ring's stream without
    /// waiting for the stream: the words go through the pinned staging buffer, whose previous
    /// copy (recorded by stage_ev, enqueued by an earlier call) must have been consumed first.
    /// A host-blocking import here would stall the host until all earlier work is done, and the
    /// GPU would then idle while the call's remaining launches are issued.
    void upload_async(void* dst, const int64_t* src, size_t n) {
        const size_t bytes = n * 8;
        if (bytes == 0) return;
        cudaStream_t st = stream_of(ctx);
        if (stage_ev) CK(cuda_check(cudaEventSynchronize(stage_ev), "staging buffer reuse"));
        else CK(cuda_check(cudaEventCreateWithFlags(&stage_ev, cudaEventDisableTiming), "staging event"));
        if (bytes > stage_bytes) {
            if (stage) cudaFreeHost(stage);
            stage = nullptr, stage_bytes = 0;
            count_alloc();
            CK(cuda_check(cudaMallocHost(&stage, bytes), "pinned staging allocation"));
            stage_bytes = bytes;
        }
        std::memcpy(stage, src, bytes);
        CK(cuda_check(cudaMemcpyAsync(dst, stage, bytes, cudaMemcpyHostToDevice, st), "staged upload"));
        CK(cuda_check(cudaEventRecord(stage_ev, st), "staging event"));
    }

    ~hc_ring_s() {
        cudaStreamSynchronize(stream_of(ctx));
        if (stage_ev) cudaEventDestroy(stage_ev);
        if (stage) cudaFreeHost(stage);
        if (side) {
            cudaStreamSynchronize(side);
            cudaStreamDestroy(side);
        }
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        for (auto& f : factors) {
            if (f.plan_lp) hc_destroy_ntt_plan(ctx, f.plan_lp);
            if (f.plan_k) hc_destroy_ntt_plan(ctx, f.plan_k);
        }
    }

    size_t n() const { return field.deg_l; }
    int64_t dl() const { return (int64_t)field.deg_lp; }
    int64_t dk() const { return (int64_t)field.deg_k; }
    int64_t prime(size_t i) const { return factors[i].p; }
    std::vector<hc_modulus> mods(const Base& b) const {
        std::vector<hc_modulus> m;
        for (size_t i : b) m.push_back(factors[i].mod);
        return m;
    }
    KMods kmods(const Base& b) const {
        REQUIRE(b.size() <= HC_MAX_MODS, HC_ERR_UNSUPPORTED, "too many RNS factors in one base");
        KMods k;
        for (size_t j = 0; j < b.size(); j++) {
            const hc_modulus& m = factors[b[j]].mod;
            k.n[j] = m.n, k.ninv[j] = m.neg_inv_n, k.r2[j] = m.r2_mod_n, k.r3[j] = m.r3_mod_n;
        }
        return k;
    }
    int64_t max_p(const Base& b) const {
        int64_t m = 1;
        for (size_t i : b) m = std::max(m, factors[i].p);
        return m;
    }
    int64_t min_p(const Base& b) const {
        int64_t m = INT64_MAX;
        for (size_t i : b) m = std::min(m, factors[i].p);
        return b.empty() ? 1 : m;
    }
    void check_base(const Base& b) const {
        for (size_t i : b) REQUIRE(i < factors.size(), HC_ERR_ARG, "RNS factor index out of range");
    }
    /// Q(base) mod p
    int64_t q_mod(const Base& b, int64_t p) const {
        int64_t r = 1 % p;
        for (size_t i : b) r = mulm(r, factors[i].p % p, p);
        return emod(r, p);
    }
    double log2_q(const Base& b) const {
        double s = 0;
        for (size_t i : b) s += std::log2((double)factors[i].p);
        return s;
    }

    // ---------------------------------------------------------------- construction
    void add_factor(int64_t p, bool transform) {
        REQUIRE(p >= ((int64_t)1 << 40) && p <= ((int64_t)1 << 57) - 1, HC_ERR_ARG, "RNS factor size");
        Factor f;
        f.p = p;
        f.transform = transform;
        CK(hc_create_modulus(p, &f.mod));
        if (transform) {
            REQUIRE((p - 1) % (int64_t)field.rou_order() == 0, HC_ERR_ARG, "RNS factor incompatible with the field");
            std::vector<size_t> olp = field.orders(0, field.nlp), ok = field.orders(field.nlp, field.cyc.size());
            CK(hc_create_ntt_plan(ctx, &f.mod, olp.data(), olp.size(), &f.plan_lp));
            CK(hc_create_ntt_plan(ctx, &f.mod, ok.data(), ok.size(), &f.plan_k));
        }
        factors.push_back(std::move(f));
    }

    /// NTT-domain CRT kernels of one factor: Gaussian periods mod the prime, transformed by the
    /// group NTT on the GPU, inverted pointwise (src/ring.rs:1338-1415).
    void ensure_kernels(Factor& f) {
        if (f.have_kernels) return;
        const int64_t p = f.p, m = (int64_t)field.m();
        int64_t zeta = 0;
        for (int64_t c = 2;; c++) {
            zeta = powm(c, (uint64_t)((p - 1) / m), p);
            bool ok = true;
            for (uint64_t q : field.m_factors) ok = ok && powm(zeta, (uint64_t)(m / (int64_t)q), p) != 1;
            if (ok) break;
        }
        int64_t z_lp = powm(zeta, crt2(1, field.spec.m_prime, 0, field.m_k()), p);
        int64_t z_k = powm(zeta, crt2(0, field.spec.m_prime, 1, field.m_k()), p);
        auto periods = [&](int64_t zp, uint64_t order, const std::vector<uint64_t>& sub,
                           const std::vector<uint64_t>& tr) {
            std::vector<int64_t> pw(order);
            int64_t cur = 1;
            for (uint64_t i = 0; i < order; i++) pw[i] = cur, cur = mulm(cur, zp, p);
            std::vector<int64_t> out;
            for (uint64_t g : tr) {
                uint64_t gi = inv_mod_u(g, field.m());
                int64_t s = 0;
                for (uint64_t x : sub) s = (s + pw[umulm(x, gi, field.m()) % order]) % p;
                out.push_back(s);
            }
            return out;
        };
        std::vector<int64_t> k_lp =
            periods(z_lp, field.spec.m_prime, field.gal_lp, field.transversal(0, field.nlp));
        std::vector<int64_t> k_k = periods(z_k, field.m_k(), field.gal_k, field.transversal(field.nlp, field.cyc.size()));
        auto to_ntt = [&](const std::vector<int64_t>& ker, hc_ntt_plan plan, bool dim2) {
            std::vector<int64_t> h;
            for (int64_t x : ker) h.push_back(mont_repr(x, p));
            int64_t len = (int64_t)h.size();
            Tensor t(ctx, 1, 1, dim2 ? len : 1, dim2 ? 1 : len);
            CK(hc_import(ctx, t.view(), h.data(), h.size()));
            CK(hc_ntt_mont64_dim(ctx, t.view(), &plan, 1, dim2 ? HC_DIM2 : HC_DIM3));
            CK(hc_export(ctx, t.view(), h.data(), h.size()));
            for (auto& x : h) x = emod(x, p);
            return h;
        };
        f.kl = to_ntt(k_lp, f.plan_lp, true);
        f.kk = to_ntt(k_k, f.plan_k, false);
        auto invert = [&](const std::vector<int64_t>& v) {
            std::vector<int64_t> o;
            for (int64_t x : v) {
                int64_t plain = from_mont(x, p);
                REQUIRE(plain != 0, HC_ERR_ARG, "CRT kernel is not invertible");
                o.push_back(mont_repr(invm(plain, p), p));
            }
            return o;
        };
        f.ikl = invert(f.kl);
        f.ikk = invert(f.kk);
        f.have_kernels = true;
    }

    TransformCache& transform_cache(const Base& b) {
        for (auto& c : tcache)
            if (c->base == b) return *c;
        check_base(b);
        auto c = std::make_unique<TransformCache>();
        c->base = b;
        c->mods = mods(b);
        std::vector<int64_t> kl, kk, ikl, ikk;
        for (size_t i : b) {
            Factor& f = factors[i];
            REQUIRE(f.transform, HC_ERR_ARG, "RNS factor doesn't support the basis transforms");
            ensure_kernels(f);
            c->plp.push_back(f.plan_lp);
            c->pk.push_back(f.plan_k);
            kl.insert(kl.end(), f.kl.begin(), f.kl.end());
            kk.insert(kk.end(), f.kk.begin(), f.kk.end());
            ikl.insert(ikl.end(), f.ikl.begin(), f.ikl.end());
            ikk.insert(ikk.end(), f.ikk.begin(), f.ikk.end());
        }
        int64_t r = (int64_t)b.size();
        auto up = [&](Tensor& t, const std::vector<int64_t>& v, bool lp) {
            t = Tensor(ctx, 1, r, lp ? dl() : 1, lp ? 1 : dk());
            CK(hc_import(ctx, t.view(), v.data(), v.size()));
        };
        up(c->kl, kl, true);
        up(c->kk, kk, false);
        up(c->ikl, ikl, true);
        up(c->ikk, ikk, false);
        tcache.push_back(std::move(c));
        return *tcache.back();
    }

    // ---------------------------------------------------------------- transforms
    /// The two fused launches of a transform (csrc/crt_fused.cu: both dimensions' NTTs of each
    /// half in one cluster launch) where the plans are the fused shapes; false: nothing was
    /// launched, the caller runs the per-dimension calls.
    bool fused_transform(TransformCache& c, const hc_view& v, bool inverse, const hc_view* post_mul,
                         const hc_view* src) {
        const size_t r = c.base.size();
        if (v.strides[3] != 1 || (src && src->strides[3] != 1)) return false;
        // broadcast view of a multiplier m over v's shape (the HAL's length-1 rule)
        auto bcast = [&](const hc_view& m, KView* out) {
            *out = kv(m);
            int64_t* st[3] = {&out->s0, &out->s1, &out->s2};
            for (int d = 0; d < 4; d++) {
                if (m.shape[d] == v.shape[d]) continue;
                if (m.shape[d] != 1) return false;
                if (d < 3) *st[d] = 0;
                else out->b3 = 1;
            }
            return m.strides[3] == 1 || m.shape[3] == 1;
        };
        KView m2{}, m3{}, pm{};
        if (!bcast(inverse ? c.ikl.view() : c.kl.view(), &m2) || !bcast(inverse ? c.ikk.view() : c.kk.view(), &m3))
            return false;
        if (post_mul && !bcast(*post_mul, &pm)) return false;
        const KView t = kv(v);
        KView sv;
        const KView* sp = nullptr;
        bool copy_first = false;
        if (src && src->ptr != v.ptr) {
            for (int d = 0; d < 4; d++)
                if (src->shape[d] != v.shape[d]) return false;
            // a source that overlaps the destination other than exactly is copied first
            auto range = [](const hc_view& x, const char** lo, const char** hi) {
                int64_t last = 0;
                for (int d = 0; d < 4; d++) last += (x.shape[d] > 0 ? x.shape[d] - 1 : 0) * (d == 3 ? 1 : x.strides[d]);
                *lo = (const char*)x.ptr;
                *hi = (const char*)x.ptr + 8 * (last + 1);
            };
            const char *dlo, *dhi, *slo, *shi;
            range(v, &dlo, &dhi);
            range(*src, &slo, &shi);
            copy_first = slo < dhi && dlo < shi;
            sv = kv(*src);
            sp = copy_first ? nullptr : &sv;
        }
        const KMods km = kmods(c.base);
        if (!crt_pass_ready(ctx, c.plp.data(), c.pk.data(), r, t)) return false;
        if (copy_first) CK(hc_assign(ctx, v, *src));
        CK(launch_crt_pass(ctx, 0, t, sp, c.plp.data(), c.pk.data(), r, m2, m3, false, km));
        CK(launch_crt_pass(ctx, 1, t, nullptr, c.plp.data(), c.pk.data(), r, KView(), pm, post_mul != nullptr, km));
        return true;
    }

    /// pb_to_crt / crt_to_pb (src/ring.rs:1118-1161); `post_mul`: a Montgomery product applied to
    /// the result in the epilogue of the last pass (the caller's next hal_mul_mont64, fused);
    /// `src`: transform a copy of src into v (the caller's hal_assign, folded into the first pass)
    void transform(const hc_view& v, const Base& b, bool inverse, const hc_view* post_mul = nullptr,
                   const hc_view* src = nullptr) {
        REQUIRE(v.shape[1] == (int64_t)b.size() && v.shape[2] == dl() && v.shape[3] == dk(), HC_ERR_SHAPE,
                "transform: tensor shape does not match the ring and base");
        TransformCache& c = transform_cache(b);
        const size_t r = b.size();
        if (fused_transform(c, v, inverse, post_mul, src)) return;
        if (src)
            CK(ntt_mul_mont64_dim_from(ctx, v, *src, c.plp.data(), r, HC_DIM2, inverse ? c.ikl.view() : c.kl.view(),
                                       c.mods.data(), r));
        else
            CK(hc_ntt_mul_mont64_dim(ctx, v, c.plp.data(), r, HC_DIM2, inverse ? c.ikl.view() : c.kl.view(),
                                     c.mods.data(), r));
        CK(hc_ntt_mul_mont64_dim(ctx, v, c.pk.data(), r, HC_DIM3, inverse ? c.ikk.view() : c.kk.view(),
                                 c.mods.data(), r));
        CK(hc_intt_mont64_dim(ctx, v, c.plp.data(), r, HC_DIM2));
        if (post_mul) CK(intt_mul_mont64_dim(ctx, v, c.pk.data(), r, HC_DIM3, *post_mul, c.mods.data(), r));
        else CK(hc_intt_mont64_dim(ctx, v, c.pk.data(), r, HC_DIM3));
    }

    // ---------------------------------------------------------------- base conversion
    BconvCache& bconv_cache(const Base& src, const Base& dst) {
        for (auto& c : bcache)
            if (c->src == src && c->dst == dst) return *c;
        check_base(src);
        check_base(dst);
        REQUIRE(!src.empty(), HC_ERR_ARG, "empty source base");
        auto c = std::make_unique<BconvCache>();
        c->src = src, c->dst = dst;
        const size_t r = src.size(), rd = dst.size();
        int64_t mx = std::max(max_p(src), max_p(dst)), mn = min_p(src);
        const int shift = (int)std::max<size_t>(64, bitlen_u128((u128)(4 * (i128)r * mx + 1)));
        REQUIRE(shift <= 126, HC_ERR_UNSUPPORTED, "base conversion precision");
        const i128 qt = (i128)1 << shift;
        REQUIRE((qt - 1) / mn + 1 <= INT64_MAX, HC_ERR_ARG, "correction vector coefficients don't fit into an i64");
        const int chunk = (int)std::min<i128>(I128MAX / ((i128)mx * mx), 1 << 30);
        std::vector<int64_t> qinv(r), mat((rd + 1) * r), qm(rd);
        for (size_t u = 0; u < r; u++) {
            int64_t pu = prime(src[u]), qo = 1;
            for (size_t l = 0; l < r; l++)
                if (l != u) qo = mulm(qo, prime(src[l]) % pu, pu);
            qinv[u] = centred(invm(qo, pu), pu);
        }
        for (size_t j = 0; j < rd; j++) {
            int64_t pj = prime(dst[j]);
            int64_t r1 = mont_repr(1, pj), r2 = mulm(r1, r1, pj);
            for (size_t u = 0; u < r; u++) {
                int64_t v = 1;
                for (size_t l = 0; l < r; l++)
                    if (l != u) v = mulm(v, prime(src[l]) % pj, pj);
                mat[j * r + u] = centred(mulm(emod(v, pj), emod(r2, pj), pj), pj);
            }
            qm[j] = centred(mulm(q_mod(src, pj), emod(-r1, pj), pj), pj);
        }
        for (size_t u = 0; u < r; u++) {
            i128 a = qt, bp = prime(src[u]);
            mat[rd * r + u] = (int64_t)((a + bp / 2) / bp);
        }
        build_bconv_tables(ctx, c->t, qinv, mods(src), mat, qm, mods(dst), {0, (int32_t)r}, shift, chunk);
        bcache.push_back(std::move(c));
        return *bcache.back();
    }

    /// `sub_mul` (optional, [2][rd]: one Montgomery factor b per destination prime, then b times
    /// -p^-1 mod 2^64): instead of writing the conversion v, dst <- mul_mont(dst - v, b) (the
    /// caller's hal_sub_i64 and hal_mul_mont64, fused into the store)
    void bconv(const hc_view& dst, const Base& db, const hc_view& src, const Base& sb,
               const int64_t* sub_mul = nullptr) {
        check_view(src, src.shape[0], (int64_t)sb.size(), src.shape[2], src.shape[3], "bconv src");
        check_view(dst, src.shape[0], (int64_t)db.size(), src.shape[2], src.shape[3], "bconv dst");
        BconvCache& c = bconv_cache(sb, db);
        CK(launch_bconv_fused(ctx, kv(src), kv(dst), c.t.c, (int)sb.size(), (int)db.size(), 1, kmods(sb), kmods(db),
                              src.shape[0], sub_mul));
    }

    GadgetCache& gadget_cache(const Base& b, const Digits& digits) {
        for (auto& c : gcache)
            if (c->base == b && c->digits == digits) return *c;
        check_base(b);
        const size_t r = b.size(), d = digits.size();
        REQUIRE(d > 0, HC_ERR_ARG, "at least one gadget digit required");
        for (size_t i = 0; i < d; i++) {
            REQUIRE(digits[i].first < digits[i].second && digits[i].second <= r, HC_ERR_ARG, "gadget digit range");
            REQUIRE(i == 0 || digits[i - 1].second <= digits[i].first, HC_ERR_ARG,
                    "digits must be sorted and disjoint");
        }
        auto c = std::make_unique<GadgetCache>();
        c->base = b, c->digits = digits;
        int64_t mx = max_p(b), mn = min_p(b);
        size_t maxlen = 0;
        for (auto& dg : digits) maxlen = std::max(maxlen, dg.second - dg.first);
        const int shift = (int)std::max<size_t>(64, bitlen_u128((u128)(4 * (i128)maxlen * mx + 1)));
        const i128 qt = (i128)1 << shift;
        REQUIRE((qt - 1) / mn + 1 <= INT64_MAX, HC_ERR_ARG, "correction vector coefficients don't fit into an i64");
        const int chunk = (int)std::min<i128>(I128MAX / ((i128)mx * mx), 1 << 30);
        auto dover = [&](size_t di, size_t u, int64_t q) {
            int64_t v = 1;
            for (size_t l = digits[di].first; l < digits[di].second; l++)
                if (l != u) v = mulm(v, prime(b[l]) % q, q);
            return emod(v, q);
        };
        std::vector<int64_t> dinv(r, 0), mat(d * (r + 1) * r, 0), dm;
        std::vector<int32_t> uc;
        for (size_t di = 0; di < d; di++) {
            uc.push_back((int32_t)digits[di].first);
            uc.push_back((int32_t)digits[di].second);
            for (size_t u = digits[di].first; u < digits[di].second; u++) {
                int64_t pu = prime(b[u]);
                dinv[u] = centred(invm(dover(di, u, pu), pu), pu);
            }
            for (size_t j = 0; j < r; j++) {
                int64_t pj = prime(b[j]);
                int64_t r1 = mont_repr(1, pj), r2 = emod(mulm(r1, r1, pj), pj);
                for (size_t u = digits[di].first; u < digits[di].second; u++)
                    mat[(di * (r + 1) + j) * r + u] = centred(mulm(dover(di, u, pj), r2, pj), pj);
                int64_t dmod = 1;
                for (size_t l = digits[di].first; l < digits[di].second; l++) dmod = mulm(dmod, prime(b[l]) % pj, pj);
                dm.push_back(centred(mulm(emod(dmod, pj), emod(-r1, pj), pj), pj));
            }
            for (size_t u = digits[di].first; u < digits[di].second; u++) {
                i128 bp = prime(b[u]);
                mat[(di * (r + 1) + r) * r + u] = (int64_t)((qt + bp / 2) / bp);
            }
        }
        build_bconv_tables(ctx, c->t, dinv, mods(b), mat, dm, mods(b), uc, shift, chunk);
        gcache.push_back(std::move(c));
        return *gcache.back();
    }

    /// src [B, r] -> dst [B d, r] (row i d + t: digit t of source i)
    void bconv_gadget(const hc_view& dst, const hc_view& src, const Base& b, const Digits& digits) {
        check_view(src, src.shape[0], (int64_t)b.size(), src.shape[2], src.shape[3], "gadget src");
        check_view(dst, src.shape[0] * (int64_t)digits.size(), (int64_t)b.size(), src.shape[2], src.shape[3],
                   "gadget dst");
        GadgetCache& c = gadget_cache(b, digits);
        KMods km = kmods(b);
        CK(launch_bconv_fused(ctx, kv(src), kv(dst), c.t.c, (int)b.size(), (int)b.size(), (int)digits.size(), km, km,
                              src.shape[0], nullptr));
    }

    // ---------------------------------------------------------------- Galois
    PermCache& perms(uint64_t g) {
        std::vector<size_t> s = field.gal_to_shift(g);
        auto it = pcache.find(s);
        if (it != pcache.end()) return *it->second;
        auto make = [&](size_t from, size_t to) {
            std::vector<size_t> sh(s.begin() + from, s.begin() + to), ord = field.orders(from, to);
            size_t n = 1;
            for (size_t o : ord) n *= o;
            std::vector<uint32_t> perm(n);
            std::vector<size_t> idx(ord.size(), 0);
            for (size_t e = 0; e < n; e++) {
                size_t src = 0;
                for (size_t t = 0; t < ord.size(); t++) src = src * ord[t] + (idx[t] + ord[t] - sh[t] % ord[t]) % ord[t];
                perm[e] = (uint32_t)src;
                for (size_t t = ord.size(); t-- > 0;) {
                    if (++idx[t] < ord[t]) break;
                    idx[t] = 0;
                }
            }
            return perm;
        };
        auto c = std::make_unique<PermCache>();
        std::vector<uint32_t> a = make(0, field.nlp), bb = make(field.nlp, field.cyc.size());
        c->p2 = DBuf(ctx, a.data(), a.size() * 4);
        c->p3 = DBuf(ctx, bb.data(), bb.size() * 4);
        auto& ref = *c;
        pcache[s] = std::move(c);
        return ref;
    }
    void apply_galois(const hc_view& dst, const hc_view& src, uint64_t g) {
        check_view(dst, src.shape[0], src.shape[1], dl(), dk(), "galois dst");
        check_view(src, dst.shape[0], dst.shape[1], dl(), dk(), "galois src");
        PermCache& pc = perms(g);
        CK(launch_galois(ctx, kv(dst), kv(src), pc.p2.as<uint32_t>(), pc.p3.as<uint32_t>()));
    }

    // ---------------------------------------------------------------- scalars
    const int64_t* one_dev(const Base& b) {
        auto it = one_cache.find(b);
        if (it != one_cache.end()) return it->second->as<int64_t>();
        std::vector<int64_t> v;
        for (size_t i : b) v.push_back(mont_repr(1, prime(i)));
        auto buf = std::make_unique<DBuf>(ctx, v.data(), v.size() * 8);
        const int64_t* p = buf->as<int64_t>();
        one_cache[b] = std::move(buf);
        return p;
    }
    /// [1, r, 1, 1] tensor of mont(scalar mod p) (src/ring.rs:876-887)
    const Tensor& scalar_tensor(const Base& b, i128 s) {
        auto key = std::make_pair(b, s);
        auto it = scalar_cache.find(key);
        if (it != scalar_cache.end()) return *it->second;
        std::vector<int64_t> v;
        for (size_t i : b) v.push_back(mont_repr((int64_t)(s % (i128)prime(i)), prime(i)));
        auto t = std::make_unique<Tensor>(ctx, 1, (int64_t)b.size(), 1, 1);
        CK(hc_import(ctx, t->view(), v.data(), v.size()));
        auto& ref = *t;
        scalar_cache[key] = std::move(t);
        return ref;
    }
    /// [1, |of|, 1, 1] tensor of mont(smallest_lift(Q(div)^-1 mod p)) for p in `of`
    /// (inverse_scalar_tensor, src/ring.rs:1165-1177), cached
    const Tensor& inv_modulus_tensor(const Base& of, const Base& div) {
        auto key = std::make_pair(of, div);
        auto it = qinv_cache.find(key);
        if (it != qinv_cache.end()) return *it->second;
        auto t = std::make_unique<Tensor>(scalar_tensor_big(of, [&](int64_t p) { return invm(q_mod(div, p), p); }));
        auto& ref = *t;
        qinv_cache[key] = std::move(t);
        return ref;
    }
    /// The factors of inv_modulus_tensor(of, div) as the base conversion's `sub_mul` pairs:
    /// [2][|of|] = (b_j, b_j * (-p_j^-1) mod 2^64), cached
    const DBuf& inv_modulus_pairs(const Base& of, const Base& div) {
        auto key = std::make_pair(of, div);
        auto it = qinv_pair_cache.find(key);
        if (it != qinv_pair_cache.end()) return *it->second;
        std::vector<int64_t> v(2 * of.size());
        for (size_t j = 0; j < of.size(); j++) {
            const int64_t p = prime(of[j]);
            v[j] = mont_repr(centred(invm(q_mod(div, p), p), p), p);
            v[of.size() + j] = (int64_t)((uint64_t)v[j] * (uint64_t)factors[of[j]].mod.neg_inv_n);
        }
        auto t = std::make_unique<DBuf>(ctx, v.data(), v.size() * 8);
        auto& ref = *t;
        qinv_pair_cache[key] = std::move(t);
        return ref;
    }
    /// [1, r, 1, 1] tensor holding mont(smallest_lift(residue(p))) (src/ring.rs:890-902)
    Tensor scalar_tensor_big(const Base& b, const std::function<int64_t(int64_t)>& residue) {
        std::vector<int64_t> v;
        for (size_t i : b) v.push_back(mont_repr(centred(residue(prime(i)), prime(i)), prime(i)));
        Tensor t(ctx, 1, (int64_t)b.size(), 1, 1);
        CK(hc_import(ctx, t.view(), v.data(), v.size()));
        return t;
    }
};

namespace {

// ------------------------------------------------------------------------- wide accumulation
/// Delayed-reduction i128 accumulator (WideRingEls, src/ring.rs:330-532): the per-row
/// worst-case bound decides between single and double reduction when finishing, and a row's
/// first accumulation overwrites it. Used for key generation and encryption (set-up work).
struct Wide {
    hc_ring R;
    Base base;
    Tensor data;
    std::vector<u128> bound;
    int64_t maxp, minp;
    Wide(hc_ring r, int64_t count, const Base& b) : R(r), base(b), bound((size_t)count, 0) {
        data = Tensor(R->ctx, count, (int64_t)b.size(), R->dl(), R->dk(), true);
        maxp = R->max_p(b), minp = R->min_p(b);
    }
    void step(size_t rs, size_t re, u128 s) {
        for (size_t i = rs; i < re; i++) {
            u128 nb = bound[i] + s;
            REQUIRE(nb >= bound[i] && nb <= (u128)I128MAX, HC_ERR_ARG, "wide ring element overflow");
            bound[i] = nb;
        }
    }
    void accumulate(size_t rs, size_t re, const hc_view& lhs, const hc_view& rhs) {
        auto op = [&](const hc_view& t, size_t s, size_t e) { return t.shape[0] == 1 ? t : vrows(t, s - rs, e - rs); };
        size_t s = rs;
        while (s < re) {
            bool fresh = bound[s] == 0;
            size_t e = s + 1;
            while (e < re && (bound[e] == 0) == fresh) e++;
            hc_view d = vrows(data.view(), (int64_t)s, (int64_t)e, true);
            if (fresh) CK(hc_mul_i64(R->ctx, d, op(lhs, s, e), op(rhs, s, e)));
            else CK(hc_fma_i64(R->ctx, d, op(lhs, s, e), op(rhs, s, e)));
            s = e;
        }
    }
    u128 mp2() const { return (u128)maxp * (u128)maxp; }
    void fma(size_t rs, size_t re, const hc_view& l, u128 lb, const hc_view& r, u128 rb) {
        accumulate(rs, re, l, r);
        step(rs, re, lb * rb * mp2());
    }
    void add(size_t rs, size_t re, const hc_view& src, u128 sb) {
        accumulate(rs, re, src, R->scalar_tensor(base, 1).view());
        step(rs, re, sb * mp2());
    }
    /// lhs any i64 tensor, rhs bounded by max_p (src/ring.rs:488-493)
    void fma_unbounded(size_t rs, size_t re, const hc_view& l, const hc_view& r) {
        accumulate(rs, re, l, r);
        step(rs, re, (u128)maxp << 63);
    }
    bool full(size_t row) const { return bound[row] > ((u128)minp << 63); }
    /// wide[rs..re) = sum_t lhs_t * rhs_t (fresh rows only; src/ring.rs:460-485), all operands
    /// almost reduced (bound 1)
    void inner_product(size_t rs, size_t re, const std::vector<hc_view>& lhs, const std::vector<hc_view>& rhs) {
        for (size_t i = rs; i < re; i++) REQUIRE(bound[i] == 0, HC_ERR_ARG, "inner product into a used row");
        REQUIRE(!lhs.empty() && lhs.size() == rhs.size(), HC_ERR_ARG, "inner product terms");
        CK(hc_inner_product_i64(R->ctx, vrows(data.view(), (int64_t)rs, (int64_t)re, true), lhs.data(), rhs.data(),
                                lhs.size()));
        step(rs, re, (u128)lhs.size() * mp2());
    }
    void reduce_into(const hc_view& dst) { reduce_rows_into(dst, bound.size()); }
    /// reduces rows [0, rows) into dst (src/ring.rs:846-865)
    void reduce_rows_into(const hc_view& dst, size_t rows) {
        std::vector<hc_modulus> m = R->mods(base);
        size_t s = 0;
        while (s < rows) {
            bool f = full(s);
            size_t e = s + 1;
            while (e < rows && full(e) == f) e++;
            hc_view d = vrows(dst, (int64_t)s, (int64_t)e);
            hc_view w = vrows(data.view(), (int64_t)s, (int64_t)e, true);
            if (f) {
                CK(hc_red_mont64_double(R->ctx, d, w, m.data(), m.size()));
                CK(hc_i64_to_mont64(R->ctx, d, m.data(), m.size()));
            } else {
                CK(hc_red_mont64(R->ctx, d, w, m.data(), m.size()));
            }
            s = e;
        }
    }
};

uint64_t splitmix(uint64_t* s) {
    *s += 0x9E3779B97F4A7C15ull;
    uint64_t z = *s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

Base base_of(const size_t* b, size_t r) {
    REQUIRE(r == 0 || b, HC_ERR_ARG, "null base");
    return Base(b, b + r);
}
Base prefix(size_t r) {
    Base b;
    for (size_t i = 0; i < r; i++) b.push_back(i);
    return b;
}
Digits digits_of(const size_t* d, size_t n) {
    REQUIRE(n == 0 || d, HC_ERR_ARG, "null digits");
    Digits r;
    for (size_t i = 0; i < n; i++) r.push_back({d[2 * i], d[2 * i + 1]});
    return r;
}
Digits clip(const Digits& d, size_t len) {
    Digits r;
    for (auto& x : d)
        if (x.first < len) r.push_back({x.first, std::min(x.second, len)});
    return r;
}
i128 words(const int64_t t[2]) { return (i128)(((u128)(uint64_t)t[1] << 64) | (uint64_t)t[0]); }

/// Tensor of element rows built on the host: mont(c mod p) for i128 coefficients c (src/ring.rs:1449-1461)
Tensor element_from_coeffs(hc_ring R, const Base& b, const std::vector<i128>& coeffs) {
    std::vector<int64_t> v;
    v.reserve(b.size() * coeffs.size());
    for (size_t i : b) {
        int64_t p = R->prime(i);
        for (i128 c : coeffs) v.push_back(mont_repr((int64_t)(c % (i128)p), p));
    }
    Tensor t(R->ctx, 1, (int64_t)b.size(), R->dl(), R->dk());
    CK(hc_import(R->ctx, t.view(), v.data(), v.size()));
    return t;
}

// ------------------------------------------------------------------------- BFV
const double MIN_SIGMA = 3.2;

double sigma_for(hc_ring R, const Base& b, double log2_alpha) {
    return std::fmax(MIN_SIGMA, std::exp2(R->log2_q(b) - log2_alpha));
}

i128 gaussian(uint64_t* st, double sigma) {
    double u1 = ((double)(splitmix(st) >> 11) + 0.5) / (double)(1ull << 53);
    double u2 = (double)(splitmix(st) >> 11) / (double)(1ull << 53);
    double g = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    return (i128)std::round(g * sigma);
}

/// b <- b + e for a fresh Gaussian e (src/bfv.rs:195-204), b in period basis
void add_error(hc_ring R, const hc_view& b, const Base& base, uint64_t* st, double sigma) {
    std::vector<i128> e(R->n());
    for (auto& x : e) x = gaussian(st, sigma);
    Tensor err = element_from_coeffs(R, base, e);
    Wide acc(R, 1, base);
    acc.add(0, 1, b, 1);
    acc.add(0, 1, err.view(), 1);
    acc.reduce_into(b);
}

/// (b + a s, -a) for uniform a (src/bfv.rs:310-326)
void finish_enc(hc_ring R, const Base& base, const hc_view& sk, const hc_view& b, uint64_t* st, const hc_view& ct) {
    std::vector<int64_t> vals;
    for (size_t i : base) {
        int64_t p = R->prime(i);
        for (size_t c = 0; c < R->n(); c++) vals.push_back((int64_t)(splitmix(st) % (uint64_t)p));
    }
    Tensor a(R->ctx, 1, (int64_t)base.size(), R->dl(), R->dk());
    CK(hc_import(R->ctx, a.view(), vals.data(), vals.size()));
    Wide acc(R, 1, base);
    acc.fma(0, 1, a.view(), 1, vbase(sk, 0, (int64_t)base.size()), 1);
    acc.add(0, 1, b, 1);
    acc.reduce_into(vrows(ct, 0, 1));
    std::vector<hc_modulus> m = R->mods(base);
    CK(hc_mul_mont64(R->ctx, a.view(), R->scalar_tensor(base, -1).view(), m.data(), m.size()));
    CK(hc_assign(R->ctx, vrows(ct, 1, 2), a.view()));
}

void enc_zero(hc_ring R, const Base& base, const hc_view& sk, uint64_t* st, double log2_alpha, const hc_view& ct) {
    Tensor b(R->ctx, 1, (int64_t)base.size(), R->dl(), R->dk());
    add_error(R, b.view(), base, st, sigma_for(R, base, log2_alpha));
    R->transform(b.view(), base, false);
    finish_enc(R, base, sk, b.view(), st, ct);
}

/// Delta = round(Q/t) modulo p (src/bfv.rs:237-247), Q = 0 mod p; ties round away from zero
std::function<int64_t(int64_t)> delta_residue(hc_ring R, const Base& base, u128 t) {
    u128 qt = 1 % t;
    for (size_t i : base) qt = (qt % t) * ((u128)R->prime(i) % t) % t;
    u128 extra = (qt + t / 2) / t;
    return [qt, t, extra](int64_t p) {
        int64_t c = (int64_t)(qt % (u128)p);
        return emod(mulm(emod(-c, p), invm((int64_t)(t % (u128)p), p), p) + (int64_t)extra, p);
    };
}

i128 cmod_t(i128 a, i128 t) {
    i128 h = t / 2, r = a % t;
    i128 ar = r < 0 ? -r : r;
    if (ar >= h) {
        if (r < 0) r += t;
        else if (r > h) r -= t;
    }
    return r;
}

void gen_ksk(hc_ring R, const Base& base, const hc_view& old_sk, const hc_view& new_sk, const Digits& digits,
             uint64_t* st, double log2_alpha, const hc_view& keys) {
    const int64_t r = (int64_t)base.size();
    check_view(keys, 2 * (int64_t)digits.size(), r, R->dl(), R->dk(), "key tensor");
    for (size_t di = 0; di < digits.size(); di++) {
        hc_view ct = vrows(keys, 2 * (int64_t)di, 2 * (int64_t)di + 2);
        enc_zero(R, base, new_sk, st, log2_alpha, ct);
        std::map<int64_t, int64_t> res;
        for (size_t j = 0; j < base.size(); j++)
            res[R->prime(base[j])] = (j >= digits[di].first && j < digits[di].second) ? 1 : 0;
        Tensor factor = R->scalar_tensor_big(base, [&res](int64_t p) { return res.at(p); });
        Wide acc(R, 1, base);
        acc.fma(0, 1, vbase(old_sk, 0, r), 1, factor.view(), 1);
        acc.add(0, 1, vrows(ct, 0, 1), 1);
        acc.reduce_into(vrows(ct, 0, 1));
    }
}

/// rows needing the full double reduction after accumulating `step_bound` (src/ring.rs:365)
bool needs_full(u128 bound, int64_t minp) { return bound > ((u128)minp << 63); }

/// gadget_decompose (src/bfv.rs:408-426): digits of B period-basis elements, in CRT basis
Tensor gadget_decompose(hc_ring R, const hc_view& c_pb, const Base& base, const Digits& digits) {
    Tensor parts = temp(R->ctx, c_pb.shape[0] * (int64_t)digits.size(), (int64_t)base.size(), R->dl(), R->dk());
    R->bconv_gadget(parts.view(), c_pb, base, digits);
    R->transform(parts.view(), base, false);
    return parts;
}

/// A key-switching key for `nd` gadget digits over the first r factors: [>= 2 nd, >= r, deg_L',
/// deg_K], dimension 3 contiguous (the kernel reads every key block through these strides).
void check_keys(hc_ring R, const hc_view& keys, int64_t r, size_t nd) {
    REQUIRE(keys.shape[1] >= r && keys.shape[0] >= 2 * (int64_t)nd, HC_ERR_SHAPE, "key tensor too small");
    REQUIRE(keys.shape[2] == R->dl() && keys.shape[3] == R->dk(), HC_ERR_SHAPE,
            "key tensor: dimensions 2 and 3 must be the ring's deg_L' and deg_K");
    REQUIRE(keys.strides[3] == 1 || R->dk() <= 1, HC_ERR_SHAPE, "key tensor: dimension 3 must be contiguous");
    REQUIRE(keys.ptr, HC_ERR_ARG, "key tensor: null data");
}

/// acc[0..2] = sum_t parts[t] * key_t (+ summands through mont(1)), reduced (fused), for B
/// ciphertexts at once: parts [B d, r] (row i d + t), summand views with one row per ciphertext,
/// out [2B, r] (rows 2i, 2i + 1).
void keyswitch(hc_ring R, const hc_view& parts, const hc_view& keys, const Base& base, size_t nd,
               const hc_view* add0, const hc_view* add1, const hc_view& out, const uint32_t* p2 = nullptr,
               const uint32_t* p3 = nullptr, bool reverse = false) {
    const int64_t r = (int64_t)base.size(), B = out.shape[0] / 2;
    check_keys(R, keys, r, nd);
    REQUIRE(parts.shape[0] == B * (int64_t)nd, HC_ERR_SHAPE, "gadget digits per ciphertext");
    // the summands have one row per ciphertext over the base, in the ring's shape
    if (add0) check_view(*add0, B, r, R->dl(), R->dk(), "key switch summand c0");
    if (add1) check_view(*add1, B, r, R->dl(), R->dk(), "key switch summand c1");
    std::vector<KView> pv, kvv;
    u128 mp = (u128)R->max_p(base), step = 0;
    for (size_t t = 0; t < nd; t++) {
        pv.push_back(kv(vstep(parts, (int64_t)t, (int64_t)nd, B)));
        kvv.push_back(kv(vbase(vrows(keys, 2 * (int64_t)t, 2 * (int64_t)t + 2), 0, r)));
        step += mp * mp;
    }
    u128 b0 = step + (add0 ? mp * mp : 0), b1 = step + (add1 ? mp * mp : 0);
    KView a0 = add0 ? kv(*add0) : KView(), a1 = add1 ? kv(*add1) : KView();
    int64_t minp = R->min_p(base);
    CK(launch_keyswitch(R->ctx, pv.data(), kvv.data(), (int)nd, add0 ? &a0 : nullptr, add1 ? &a1 : nullptr,
                        needs_full(b0, minp), needs_full(b1, minp), kv(out), R->kmods(base), R->one_dev(base), p2, p3,
                        reverse));
}

/// Independent work of one call on the ring's side stream: begin() orders the branch after the
/// current stream's prior work and makes the side stream current, back() makes the original stream
/// current again while the branch keeps running, join() makes the original stream wait for the
/// branch (device-side; the host does not block). Inside a graph capture the branch becomes a
/// parallel path of the graph. The destructor restores the original stream and joins on every
/// exit path.
struct SideBranch {
    hc_ring R;
    void* main;
    bool on_side = false, open = false;
    explicit SideBranch(hc_ring r) : R(r), main(hc_context_stream(r->ctx)) {}
    void begin() {
        CK(cuda_check(cudaEventRecord(R->fork_ev, (cudaStream_t)main), "branch fork"));
        CK(cuda_check(cudaStreamWaitEvent(R->side, R->fork_ev, 0), "branch fork"));
        CK(hc_context_set_stream(R->ctx, R->side));
        on_side = open = true;
    }
    void back() {
        CK(hc_context_set_stream(R->ctx, main));
        on_side = false;
    }
    void join() {
        if (on_side) back();
        if (!open) return;
        open = false;
        CK(cuda_check(cudaEventRecord(R->join_ev, R->side), "branch join"));
        CK(cuda_check(cudaStreamWaitEvent((cudaStream_t)main, R->join_ev, 0), "branch join"));
    }
    ~SideBranch() {
        if (on_side) hc_context_set_stream(R->ctx, main);
        if (open) {
            cudaEventRecord(R->join_ev, R->side);
            cudaStreamWaitEvent((cudaStream_t)main, R->join_ev, 0);
        }
    }
    SideBranch(const SideBranch&) = delete;
    SideBranch& operator=(const SideBranch&) = delete;
};

/// The extension base of lift_to_extended (src/bfv.rs:564-598, src/ring.rs:716-731): extension
/// primes until log2 Q + t_bits + 60 bits are covered.
Base extension_of(hc_ring R, const Base& base) {
    Base ext;
    double need = (double)(product_bits([&] {
                               std::vector<int64_t> ps;
                               for (size_t i : base) ps.push_back(R->prime(i));
                               return ps;
                           }()) +
                           R->t_bits + 60);
    double bits = 0;
    for (size_t i = R->initial_len; i < R->factors.size() && bits < need; i++) {
        ext.push_back(i);
        bits += std::log2((double)R->prime(i));
    }
    REQUIRE(bits >= need, HC_ERR_ARG, "extension pool too small for lifted multiplication over this base");
    return ext;
}

/// The extension rows of lift_to_extended for a CRT-basis input whose period-basis form is pb:
/// [count, |ext|] in CRT basis (the base rows would be the input itself).
Tensor lift_extension_rows(hc_ring R, const hc_view& pb, const Base& base, const Base& ext) {
    Tensor hi = temp(R->ctx, pb.shape[0], (int64_t)ext.size(), R->dl(), R->dk());
    R->bconv(hi.view(), ext, pb, base);
    R->transform(hi.view(), ext, false);
    return hi;
}

Tensor lift_to_extended(hc_ring R, const hc_view& pb, const hc_view* crt, const Base& base) {
    const int64_t count = pb.shape[0], r = (int64_t)base.size();
    const Base ext = extension_of(R, base);
    Base lifted = base;
    lifted.insert(lifted.end(), ext.begin(), ext.end());
    Tensor res = temp(R->ctx, count, (int64_t)lifted.size(), R->dl(), R->dk());
    hc_view hi = vbase(res.view(), r, (int64_t)lifted.size());
    R->bconv(hi, ext, pb, base);
    if (crt) {
        R->transform(hi, ext, false);
        CK(hc_assign(R->ctx, vbase(res.view(), 0, r), *crt));
    } else {
        CK(hc_assign(R->ctx, vbase(res.view(), 0, r), pb));
        R->transform(res.view(), lifted, false);
    }
    return res;
}

/// rescale_to_base (src/bfv.rs:601-622); `pre_scaled`: x was already multiplied by t (fused into
/// the epilogue of the transform that produced it)
Tensor rescale_to_base(hc_ring R, const hc_view& x, const Base& lifted, size_t base_len, i128 t,
                       bool pre_scaled = false) {
    const int64_t count = x.shape[0];
    Base base(lifted.begin(), lifted.begin() + base_len), ext(lifted.begin() + base_len, lifted.end());
    std::vector<hc_modulus> ml = R->mods(lifted);
    if (!pre_scaled) CK(hc_mul_mont64(R->ctx, x, R->scalar_tensor(lifted, t).view(), ml.data(), ml.size()));
    hc_view xlo = vbase(x, 0, (int64_t)base_len), xhi = vbase(x, (int64_t)base_len, (int64_t)lifted.size());
    // xhi <- (xhi - bconv(xlo)) * (Q_base^-1 mod p), the subtraction and product in the conversion's store
    R->bconv(xhi, ext, xlo, base, R->inv_modulus_pairs(ext, base).as<int64_t>());
    Tensor out = temp(R->ctx, count, (int64_t)base_len, R->dl(), R->dk());
    R->bconv(out.view(), base, xhi, ext);
    return out;
}

}  // namespace

extern "C" {

hc_status hc_ring_create(hc_context ctx, const char* field, size_t lo, size_t hi, size_t t_bits, hc_ring* out) {
    return guard([&] {
        REQUIRE(ctx && field && out, HC_ERR_ARG, "null argument");
        REQUIRE(hi > lo, HC_ERR_ARG, "log2 q range");
        auto R = std::make_unique<hc_ring_s>();
        R->ctx = ctx;
        R->create_side();
        R->field = Field::make(field);
        int64_t rou = (int64_t)R->field.rou_order();
        std::vector<int64_t> base = sample_primes({}, lo, hi, 57, rou);
        std::vector<int64_t> all = sample_primes(base, 2 * hi + 60 + t_bits, 2 * hi + 60 + t_bits + 30, 57, rou);
        R->initial_len = base.size();
        R->t_bits = t_bits;
        for (int64_t p : all) R->add_factor(p, true);
        *out = R.release();
    });
}

hc_status hc_ring_create_raw(hc_context ctx, const char* field, const int64_t* primes, size_t n, hc_ring* out) {
    return guard([&] {
        REQUIRE(ctx && field && out && (n == 0 || primes), HC_ERR_ARG, "null argument");
        auto R = std::make_unique<hc_ring_s>();
        R->ctx = ctx;
        R->create_side();
        R->field = Field::make(field);
        R->initial_len = n;
        for (size_t i = 0; i < n; i++) {
            for (auto& f : R->factors) REQUIRE(f.p != primes[i], HC_ERR_ARG, "duplicate RNS factor");
            R->add_factor(primes[i], false);
        }
        *out = R.release();
    });
}

hc_status hc_ring_destroy(hc_ring ring) {
    delete ring;
    return HC_OK;
}
size_t hc_ring_num_factors(hc_ring ring) { return ring ? ring->factors.size() : 0; }
int64_t hc_ring_prime(hc_ring ring, size_t idx) { return ring && idx < ring->factors.size() ? ring->factors[idx].p : 0; }
size_t hc_ring_initial_len(hc_ring ring) { return ring ? ring->initial_len : 0; }
hc_status hc_ring_dims(hc_ring ring, size_t out[3]) {
    if (!ring || !out) return fail(HC_ERR_ARG, "null argument");
    out[0] = ring->field.deg_l, out[1] = ring->field.deg_lp, out[2] = ring->field.deg_k;
    return HC_OK;
}
hc_status hc_ring_modulus(hc_ring ring, size_t idx, hc_modulus* out) {
    if (!ring || !out || idx >= ring->factors.size()) return fail(HC_ERR_ARG, "bad argument");
    *out = ring->factors[idx].mod;
    return HC_OK;
}
hc_status hc_ring_extension_base(hc_ring ring, const size_t* base, size_t r, size_t* out, size_t* out_len) {
    return guard([&] {
        REQUIRE(ring && out && out_len, HC_ERR_ARG, "null argument");
        Base b = base_of(base, r);
        for (size_t i : b) REQUIRE(i < ring->initial_len, HC_ERR_ARG, "extension of a non-initial base");
        std::vector<int64_t> ps;
        for (size_t i : b) ps.push_back(ring->prime(i));
        double need = (double)(product_bits(ps) + ring->t_bits + 60), bits = 0;
        size_t n = 0;
        for (size_t i = ring->initial_len; i < ring->factors.size() && bits < need; i++) {
            out[n++] = i;
            bits += std::log2((double)ring->prime(i));
        }
        REQUIRE(bits >= need, HC_ERR_ARG, "extension pool too small for lifted multiplication over this base");
        *out_len = n;
    });
}
hc_status hc_ring_crt_kernels(hc_ring ring, size_t idx, int64_t* out) {
    return guard([&] {
        REQUIRE(ring && out && idx < ring->factors.size(), HC_ERR_ARG, "bad argument");
        Factor& f = ring->factors[idx];
        REQUIRE(f.transform, HC_ERR_ARG, "RNS factor doesn't support the basis transforms");
        ring->ensure_kernels(f);
        size_t dl = f.kl.size(), dk = f.kk.size();
        std::memcpy(out, f.kl.data(), dl * 8);
        std::memcpy(out + dl, f.kk.data(), dk * 8);
        std::memcpy(out + dl + dk, f.ikl.data(), dl * 8);
        std::memcpy(out + 2 * dl + dk, f.ikk.data(), dk * 8);
    });
}

hc_status hc_ring_pb_to_crt(hc_ring ring, hc_view data, const size_t* base, size_t r) {
    return guard([&] {
        REQUIRE(ring, HC_ERR_ARG, "null ring");
        ring->transform(data, base_of(base, r), false);
    });
}
hc_status hc_ring_crt_to_pb(hc_ring ring, hc_view data, const size_t* base, size_t r) {
    return guard([&] {
        REQUIRE(ring, HC_ERR_ARG, "null ring");
        ring->transform(data, base_of(base, r), true);
    });
}
hc_status hc_ring_bconv(hc_ring ring, hc_view dst, const size_t* db, size_t rd, hc_view src, const size_t* sb,
                        size_t rs) {
    return guard([&] {
        REQUIRE(ring, HC_ERR_ARG, "null ring");
        ring->bconv(dst, base_of(db, rd), src, base_of(sb, rs));
    });
}
hc_status hc_ring_bconv_gadget(hc_ring ring, hc_view dst, hc_view src, const size_t* base, size_t r,
                               const size_t* digits, size_t d) {
    return guard([&] {
        REQUIRE(ring, HC_ERR_ARG, "null ring");
        ring->bconv_gadget(dst, src, base_of(base, r), digits_of(digits, d));
    });
}
hc_status hc_ring_apply_galois(hc_ring ring, hc_view dst, hc_view src, const size_t* base, size_t r, uint64_t g) {
    return guard([&] {
        REQUIRE(ring, HC_ERR_ARG, "null ring");
        REQUIRE((int64_t)r == src.shape[1], HC_ERR_SHAPE, "base length does not match the tensor");
        (void)base;  // the automorphism permutes positions; which factors the rows hold does not matter
        ring->apply_galois(dst, src, g);
    });
}

hc_status hc_bfv_gen_sk(hc_ring R, uint64_t* st, hc_view sk) {
    return guard([&] {
        REQUIRE(R && st, HC_ERR_ARG, "null argument");
        Base b = prefix(R->initial_len);
        check_view(sk, 1, (int64_t)b.size(), R->dl(), R->dk(), "sk");
        std::vector<i128> c(R->n(), 0);
        for (int i = 0; i < 128; i++) {  // SK_HWT (src/bfv.rs:41)
            size_t j = (size_t)(splitmix(st) % (uint64_t)R->n());
            c[j] = (i128)(splitmix(st) % 2) * 2 - 1;
        }
        Tensor t = element_from_coeffs(R, b, c);
        R->transform(t.view(), b, false);
        CK(hc_assign(R->ctx, sk, t.view()));
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_bfv_gen_sk_uniform_ternary(hc_ring R, uint64_t* st, hc_view sk) {
    return guard([&] {
        REQUIRE(R && st, HC_ERR_ARG, "null argument");
        Base b = prefix(R->initial_len);
        check_view(sk, 1, (int64_t)b.size(), R->dl(), R->dk(), "sk");
        std::vector<i128> c(R->n(), 0);
        for (size_t j = 0; j < R->n(); j++) c[j] = (i128)(splitmix(st) % 3) - 1;
        Tensor t = element_from_coeffs(R, b, c);
        R->transform(t.view(), b, false);
        CK(hc_assign(R->ctx, sk, t.view()));
        CK(hc_synchronize(R->ctx));
    });
}

double hc_bfv_log2_alpha_for_sigma(hc_ring R, const size_t* base, size_t r, double sigma) {
    return R->log2_q(Base(base, base + r)) - std::log2(sigma);
}

hc_status hc_bfv_enc(hc_ring R, uint64_t* st, const size_t* base, size_t r, const int64_t t[2], const int64_t* ptxt,
                     hc_view sk, double log2_alpha, hc_view ct) {
    return guard([&] {
        REQUIRE(R && st && t && ptxt, HC_ERR_ARG, "null argument");
        Base b = base_of(base, r);
        R->check_base(b);
        check_view(ct, 2, (int64_t)r, R->dl(), R->dk(), "ciphertext");
        const i128 tt = words(t);
        REQUIRE(tt >= 2, HC_ERR_ARG, "plaintext modulus");
        std::vector<i128> c(R->n());
        for (size_t i = 0; i < R->n(); i++)
            c[i] = cmod_t((i128)(((u128)(uint64_t)ptxt[2 * i + 1] << 64) | (uint64_t)ptxt[2 * i]), tt);
        Tensor bt = element_from_coeffs(R, b, c);
        std::vector<hc_modulus> m = R->mods(b);
        Tensor delta = R->scalar_tensor_big(b, delta_residue(R, b, (u128)tt));
        CK(hc_mul_mont64(R->ctx, bt.view(), delta.view(), m.data(), m.size()));
        add_error(R, bt.view(), b, st, sigma_for(R, b, log2_alpha));
        R->transform(bt.view(), b, false);
        finish_enc(R, b, sk, bt.view(), st, ct);
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_bfv_gen_ksk(hc_ring R, uint64_t* st, const size_t* base, size_t r, hc_view old_sk, hc_view new_sk,
                         const size_t* digits, size_t d, double log2_alpha, hc_view keys) {
    return guard([&] {
        REQUIRE(R && st, HC_ERR_ARG, "null argument");
        Base b = base_of(base, r);
        R->check_base(b);
        gen_ksk(R, b, old_sk, new_sk, digits_of(digits, d), st, log2_alpha, keys);
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_bfv_gen_rk(hc_ring R, uint64_t* st, hc_view sk, const size_t* digits, size_t d, double log2_alpha,
                        hc_view keys) {
    return guard([&] {
        REQUIRE(R && st, HC_ERR_ARG, "null argument");
        Base b = prefix(R->initial_len);
        Wide acc(R, 1, b);
        acc.fma(0, 1, sk, 1, sk, 1);
        Tensor sq(R->ctx, 1, (int64_t)b.size(), R->dl(), R->dk());
        acc.reduce_into(sq.view());
        gen_ksk(R, b, sq.view(), sk, digits_of(digits, d), st, log2_alpha, keys);
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_bfv_gen_gk(hc_ring R, uint64_t* st, hc_view sk, uint64_t g, const size_t* digits, size_t d,
                        double log2_alpha, hc_view keys) {
    return guard([&] {
        REQUIRE(R && st, HC_ERR_ARG, "null argument");
        Base b = prefix(R->initial_len);
        Tensor gs(R->ctx, 1, (int64_t)b.size(), R->dl(), R->dk());
        R->apply_galois(gs.view(), sk, g);
        gen_ksk(R, b, gs.view(), sk, digits_of(digits, d), st, log2_alpha, keys);
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_bfv_noisy_plaintext(hc_ring R, hc_view ct, const size_t* base, size_t r, hc_view sk, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        check_view(ct, 2, (int64_t)r, R->dl(), R->dk(), "ciphertext");
        Wide acc(R, 1, b);
        acc.fma(0, 1, vrows(ct, 1, 2), 1, vbase(sk, 0, (int64_t)r), 1);
        acc.add(0, 1, vrows(ct, 0, 1), 1);
        acc.reduce_into(out);
        R->transform(out, b, true);
    });
}

hc_status hc_bfv_key_switch(hc_ring R, hc_view c0, hc_view c1_pb, const size_t* base, size_t r, hc_view keys,
                            const size_t* digits, size_t d, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        check_view(out, 2, (int64_t)r, R->dl(), R->dk(), "key switch output");
        check_view(c0, 1, (int64_t)r, R->dl(), R->dk(), "key switch c0");
        check_view(c1_pb, 1, (int64_t)r, R->dl(), R->dk(), "key switch c1");
        Digits dg = clip(digits_of(digits, d), r);
        check_keys(R, keys, (int64_t)r, dg.size());
        Tensor parts = gadget_decompose(R, c1_pb, b, dg);
        keyswitch(R, parts.view(), keys, b, dg.size(), &c0, nullptr, out);
    });
}

hc_status hc_bfv_lift_to_extended(hc_ring R, hc_view pb, hc_view crt, const size_t* base, size_t r, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        Tensor t = lift_to_extended(R, pb, crt.ptr ? &crt : nullptr, b);
        check_view(out, t.shape[0], t.shape[1], t.shape[2], t.shape[3], "lift output");
        CK(hc_assign(R->ctx, out, t.view()));
    });
}

hc_status hc_bfv_rescale_to_base(hc_ring R, hc_view x, const size_t* base, size_t r, size_t base_len,
                                 const int64_t t[2], hc_view out) {
    return guard([&] {
        REQUIRE(R && t, HC_ERR_ARG, "null argument");
        Tensor o = rescale_to_base(R, x, base_of(base, r), base_len, words(t));
        check_view(out, o.shape[0], o.shape[1], o.shape[2], o.shape[3], "rescale output");
        CK(hc_assign(R->ctx, out, o.view()));
    });
}

hc_status hc_bfv_mod_switch_down(hc_ring R, hc_view x, const size_t* base, size_t r, size_t new_len, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        REQUIRE(new_len <= r, HC_ERR_ARG, "new length exceeds the base");
        check_view(out, x.shape[0], (int64_t)new_len, R->dl(), R->dk(), "mod switch output");
        if (new_len == r) {
            CK(hc_assign(R->ctx, out, x));
            return;
        }
        Base kept(b.begin(), b.begin() + new_len), dropped(b.begin() + new_len, b.end());
        Tensor tmp(R->ctx, x.shape[0], (int64_t)new_len, R->dl(), R->dk());
        R->bconv(tmp.view(), kept, vbase(x, (int64_t)new_len, (int64_t)r), dropped);
        CK(hc_assign(R->ctx, out, vbase(x, 0, (int64_t)new_len)));
        CK(hc_sub_i64(R->ctx, out, tmp.view()));
        const Tensor& inv = R->inv_modulus_tensor(kept, dropped);  // cached: no upload per call
        std::vector<hc_modulus> m = R->mods(kept);
        CK(hc_mul_mont64(R->ctx, out, inv.view(), m.data(), m.size()));
    });
}

hc_status hc_bfv_hom_mul(hc_ring R, const int64_t t[2], hc_view ct1, hc_view ct2, const size_t* base, size_t r,
                         hc_view rk, const size_t* digits, size_t d, int period_output, hc_view out) {
    return guard([&] {
        REQUIRE(R && t, HC_ERR_ARG, "null argument");
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r;
        REQUIRE(ct1.shape[0] >= 2 && ct1.shape[0] % 2 == 0, HC_ERR_SHAPE, "ciphertexts must have 2 rows each");
        const int64_t B = ct1.shape[0] / 2;  // independent ciphertext pairs, stacked along dimension 0
        check_view(ct1, 2 * B, rr, R->dl(), R->dk(), "ct1");
        check_view(ct2, 2 * B, rr, R->dl(), R->dk(), "ct2");
        check_view(out, 2 * B, rr, R->dl(), R->dk(), "output");
        // lift both operands (src/bfv.rs:762-768): the lifted tensors' base rows are the operands
        // themselves, so only the extension rows are formed and the tensor product reads both parts
        const Base ext = extension_of(R, b);
        auto lift = [&](const hc_view& ct) {
            Tensor pb = temp(R->ctx, 2 * B, rr, R->dl(), R->dk());
            R->transform(pb.view(), b, true, nullptr, &ct);  // pb = crt_to_pb(ct)
            return lift_extension_rows(R, pb.view(), b, ext);
        };
        // the two lifts are independent: the second runs on the side stream beside the first
        SideBranch lifts(R);
        lifts.begin();
        Tensor rh = lift(ct2);
        lifts.back();
        Tensor lh = lift(ct1);
        lifts.join();
        Base lifted = b;
        lifted.insert(lifted.end(), ext.begin(), ext.end());
        // tensor product + reduce_wide (src/bfv.rs:667-683, :769-771); rows 2i, 2i + 1 hold
        // (c0, c1) of product i and row 2B + i its c2, so that both groups are contiguous
        Tensor prod = temp(R->ctx, 3 * B, (int64_t)lifted.size(), R->dl(), R->dk());
        {
            u128 mp = (u128)R->max_p(lifted), s1 = mp * mp;
            int64_t mn = R->min_p(lifted);
            CK(launch_tensor(R->ctx, kv(prod.view()), kv(ct1), kv(lh.view()), kv(ct2), kv(rh.view()), (int)rr,
                             R->kmods(lifted), needs_full(s1, mn), needs_full(2 * s1, mn), needs_full(s1, mn)));
        }
        const Tensor& tscale = R->scalar_tensor(lifted, words(t));
        const hc_view tsv = tscale.view();
        // relinearisation (src/bfv.rs:699-741)
        Digits dg = clip(digits_of(digits, d), r);
        REQUIRE(rk.shape[0] >= 2 * (int64_t)dg.size() && rk.shape[1] >= rr, HC_ERR_SHAPE, "relinearisation key shape");
        // from here the (c0, c1) rows and the c2 rows are independent until the key switch: c2's
        // transform, rescale and gadget decomposition run on the side stream beside c0, c1's
        // transform, rescale and (CRT output) forward transform
        const hc_view p01 = vrows(prod.view(), 0, 2 * B), p2 = vrows(prod.view(), 2 * B, 3 * B);
        SideBranch c2_branch(R);
        c2_branch.begin();
        R->transform(p2, lifted, true, &tsv);
        Tensor resc2 = rescale_to_base(R, p2, lifted, r, words(t), true);
        Tensor parts = gadget_decompose(R, resc2.view(), b, dg);
        c2_branch.back();
        R->transform(p01, lifted, true, &tsv);
        Tensor resc01 = rescale_to_base(R, p01, lifted, r, words(t), true);
        const hc_view c01 = resc01.view();
        if (!period_output) R->transform(c01, b, false);
        c2_branch.join();
        if (!period_output) {
            hc_view a0 = vstep(c01, 0, 2, B), a1 = vstep(c01, 1, 2, B);
            keyswitch(R, parts.view(), rk, b, dg.size(), &a0, &a1, out);
        } else {
            keyswitch(R, parts.view(), rk, b, dg.size(), nullptr, nullptr, out);
            R->transform(out, b, true);
            CK(hc_add_i64(R->ctx, out, c01));
        }
    });
}

/// B ciphertexts [2B, r] (rows 2i, 2i + 1) under one automorphism g: the gadget decomposition and
/// the key switch each run once over the whole batch.
hc_status hc_bfv_hom_gal_batch(hc_ring R, hc_view ct, const size_t* base, size_t r, uint64_t g, hc_view gk,
                               const size_t* digits, size_t d, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r;
        REQUIRE(ct.shape[0] >= 2 && ct.shape[0] % 2 == 0, HC_ERR_SHAPE, "ciphertexts must have 2 rows each");
        const int64_t B = ct.shape[0] / 2;
        check_view(ct, 2 * B, rr, R->dl(), R->dk(), "ciphertexts");
        check_view(out, 2 * B, rr, R->dl(), R->dk(), "output");
        Digits dg = clip(digits_of(digits, d), r);
        REQUIRE(gk.shape[0] >= 2 * (int64_t)dg.size() && gk.shape[1] >= rr, HC_ERR_SHAPE, "Galois key tensor shape");
        Tensor c1(R->ctx, B, rr, R->dl(), R->dk());
        const hc_view c1_crt = vstep(ct, 1, 2, B);
        R->transform(c1.view(), b, true, nullptr, &c1_crt);
        Tensor parts = gadget_decompose(R, c1.view(), b, dg);
        hc_view c0 = vstep(ct, 0, 2, B);
        PermCache& pc = R->perms(g);
        keyswitch(R, parts.view(), gk, b, dg.size(), &c0, nullptr, out, pc.p2.as<uint32_t>(), pc.p3.as<uint32_t>());
    });
}

hc_status hc_bfv_hom_gal(hc_ring R, hc_view ct, const size_t* base, size_t r, const uint64_t* gs, size_t ngs,
                         hc_view gks, const size_t* digits, size_t d, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        if (ngs == 0) return;
        REQUIRE(gs, HC_ERR_ARG, "null automorphism list");
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r;
        check_view(ct, 2, rr, R->dl(), R->dk(), "ciphertext");
        check_view(out, 2 * (int64_t)ngs, rr, R->dl(), R->dk(), "output");
        Digits dg = clip(digits_of(digits, d), r);
        const int64_t per = 2 * (int64_t)d;
        REQUIRE(gks.shape[0] == per * (int64_t)ngs && gks.shape[1] >= rr, HC_ERR_SHAPE, "galois key tensor shape");
        Tensor c1(R->ctx, 1, rr, R->dl(), R->dk());
        const hc_view c1_crt = vrows(ct, 1, 2);
        R->transform(c1.view(), b, true, nullptr, &c1_crt);
        Tensor parts = gadget_decompose(R, c1.view(), b, dg);
        hc_view c0 = vrows(ct, 0, 1);
        for (size_t gi = 0; gi < ngs; gi++) {
            PermCache& pc = R->perms(gs[gi]);
            keyswitch(R, parts.view(), vrows(gks, per * (int64_t)gi, per * (int64_t)(gi + 1)), b, dg.size(), &c0,
                      nullptr, vrows(out, 2 * (int64_t)gi, 2 * (int64_t)gi + 2), pc.p2.as<uint32_t>(),
                      pc.p3.as<uint32_t>());
        }
    });
}

}  // extern "C"

// ------------------------------------------------------------------------- key switching without allocation
//
// hc_bfv_key_switch_noalloc is hc_bfv_key_switch for callers that must not allocate device memory:
// hosts whose device memory is handed out by their own arena or budget (a language runtime or a
// serving process that reserves HBM up front), and code paths where cudaMalloc / cudaFree are not
// permitted or would synchronise the device at the wrong moment. The only scratch it needs, the
// gadget digits of c1 (d x r x deg_L' x deg_K residues), lives in the static array below, which
// every GPU that loads this library holds until the process exits.

/// Words (i64) of the scratch array: 32 MiB per GPU.
#define HC_KS_NOALLOC_WORDS ((size_t)1 << 22)

/// Gadget digits of the no-allocation key switch. Host code never dereferences this name: its
/// device address comes from cudaGetSymbolAddress, once per device.
static __device__ __align__(256) int64_t hc_ks_noalloc_scratch[HC_KS_NOALLOC_WORDS];

namespace {

std::mutex ks_noalloc_mu;
std::map<int, int64_t*> ks_noalloc_addr;  // device ordinal -> address of the scratch array there

/// Address of the scratch array on `device`, looked up on the first call for that device with
/// the device made current for the lookup (and the caller's current device restored). It is kept
/// for the life of the process; a device reset would leave it stale, like every other device
/// object of the library, which is why no call may follow a reset.
int64_t* ks_noalloc_scratch(int device) {
    std::lock_guard<std::mutex> lock(ks_noalloc_mu);
    auto it = ks_noalloc_addr.find(device);
    if (it != ks_noalloc_addr.end()) return it->second;
    int prev = 0;
    CK(cuda_check(cudaGetDevice(&prev), "cudaGetDevice"));
    if (prev != device) CK(cuda_check(cudaSetDevice(device), "cudaSetDevice"));
    int64_t* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&p, hc_ks_noalloc_scratch);
    if (prev != device) cudaSetDevice(prev);
    CK(cuda_check(e, "address of the key-switch scratch array"));
    ks_noalloc_addr[device] = p;
    return p;
}

/// Whether the ring already holds every device table the key switch reads for this base and
/// digit split (CRT kernels, gadget conversion constants, Montgomery ones), so that no call below
/// has to build and upload one.
bool ks_tables_ready(hc_ring R, const Base& b, const Digits& dg) {
    bool t = false, g = false;
    for (auto& c : R->tcache) t = t || c->base == b;
    for (auto& c : R->gcache) g = g || (c->base == b && c->digits == dg);
    return t && g && R->one_cache.count(b) > 0;
}

}  // namespace

extern "C" hc_status hc_bfv_key_switch_noalloc(hc_ring R, hc_view c0, hc_view c1_pb, const size_t* base, size_t r,
                                               hc_view keys, const size_t* digits, size_t d, hc_view out) {
    return guard([&] {
        REQUIRE(R, HC_ERR_ARG, "null ring");
        Base b = base_of(base, r);
        check_view(out, 2, (int64_t)r, R->dl(), R->dk(), "key switch output");
        check_view(c0, 1, (int64_t)r, R->dl(), R->dk(), "key switch c0");
        check_view(c1_pb, 1, (int64_t)r, R->dl(), R->dk(), "key switch c1");
        Digits dg = clip(digits_of(digits, d), r);
        REQUIRE(!dg.empty(), HC_ERR_ARG, "at least one gadget digit required");
        check_keys(R, keys, (int64_t)r, dg.size());
        const size_t words = dg.size() * r * (size_t)R->dl() * (size_t)R->dk();
        REQUIRE(words <= HC_KS_NOALLOC_WORDS, HC_ERR_UNSUPPORTED,
                "no-allocation key switch: digits x RNS factors x ring degree = " + std::to_string(words) +
                    " exceeds the scratch array of " + std::to_string(HC_KS_NOALLOC_WORDS) + " words (32 MiB)");
        REQUIRE(ks_tables_ready(R, b, dg), HC_ERR_ARG,
                "no-allocation key switch: the ring has no tables for this base and digit split yet; any "
                "key-switching call with this base and digit split (hc_bfv_key_switch, the relinearisation of "
                "hc_bfv_hom_mul, hc_bfv_hom_gal) builds them");
        int64_t* scratch = ks_noalloc_scratch(device_of(R->ctx));
        hc_view parts;
        parts.ptr = scratch;
        parts.shape[0] = (int64_t)dg.size(), parts.shape[1] = (int64_t)r, parts.shape[2] = R->dl();
        parts.shape[3] = R->dk();
        parts.strides[3] = 1, parts.strides[2] = R->dk(), parts.strides[1] = R->dl() * R->dk();
        parts.strides[0] = (int64_t)r * R->dl() * R->dk();
        // every digit residue is written by the conversion before it is read: nothing to clear
        R->bconv_gadget(parts, c1_pb, b, dg);
        R->transform(parts, b, false);
        keyswitch(R, parts, keys, b, dg.size(), &c0, nullptr, out);
    });
}

// ------------------------------------------------------------------------- batched CRT transforms

namespace hc {
hc_status launch_crt_batch(hc_context ctx, const CrtSlab* slabs, int nslabs, int* counter, size_t tile_words,
                           size_t tw_words, const CrtLaunch& L, bool generic, int cls);
int crt_slab_kernel_class(int32_t shapes);
bool crt_slab_specialised(int32_t shapes);
const void* plan_device(hc_ntt_plan p);
int32_t plan_ntw(hc_ntt_plan p);
int32_t plan_shape(hc_ntt_plan p);
}  // namespace hc

/// The slabs of one shape class (crt_slab_class): one persistent launch with its own tuned shape.
struct CrtGroup {
    std::vector<CrtSlab> host;  // sorted: largest slabs first
    DBuf dev;                   // the descriptors on the device
    DBuf counter;               // next slab of the running launch
    size_t tw_words = 0;
    CrtLaunch launch{256, 3, 6};
    std::string signature;      // composition of the group, key of the autotuner's memory
    int64_t residues = 0;
};

struct hc_crt_batch_s {
    hc_context ctx = nullptr;
    std::vector<CrtGroup> groups;  // by shape class; groups[0] holds the most residues
};

namespace {

std::mutex crt_tune_mu;
std::map<std::string, CrtLaunch> crt_tuned;  // signature -> launch shape chosen by the autotuner

/// The group's slabs grouped by (deg_L', deg_K, ops), with their counts: groups of the same shape
/// class and composition share a tuned launch shape.
std::string crt_signature(const std::vector<CrtSlab>& v) {
    std::map<std::tuple<int, int, int>, size_t> m;
    for (const CrtSlab& s : v) m[std::make_tuple(s.dl, s.dk, s.ops)]++;
    std::string out;
    for (auto& kv : m) {
        // counts rounded to powers of two: nearby batch sizes tune alike
        size_t c = 1;
        while (c < kv.second) c <<= 1;
        out += std::to_string(std::get<0>(kv.first)) + "x" + std::to_string(std::get<1>(kv.first)) + "/" +
               std::to_string(std::get<2>(kv.first)) + ":" + std::to_string(c) + ";";
    }
    return out;
}

/// Shape class of a slab: its specialised (line, column) shapes when it has them, else 0 (the
/// generic tile programme). Slabs of one class run the same code, so a launch per class keeps
/// each kernel's working code small and lets each class have its own launch shape.
int crt_slab_class(const CrtSlab& s) { return crt_slab_specialised(s.shapes) ? (s.shapes & 0xffff) : 0; }

/// Shared-memory tile of a slab: a padded line for the specialised line kernels, else the
/// larger of a line and a column block; rounded to an even word count (16-byte aligned twiddles).
size_t crt_tile_words(const CrtSlab& s, int logv) { return crt_slab_tile_words(s.shapes, s.dl, s.dk, logv); }

/// Whether some slab needs the generic tile programme (crt_batch_kernel<true>).
bool crt_generic(const std::vector<CrtSlab>& slabs) {
    for (const CrtSlab& s : slabs)
        if (!crt_slab_specialised(s.shapes)) return true;
    return false;
}

/// The kernel class of a group's specialised slabs: their shape class when they all share one,
/// else 0 (the kernel that carries both classes' code).
int crt_group_kernel_class(const CrtGroup& g) {
    if (g.host.empty()) return 0;
    const int c = crt_slab_kernel_class(g.host[0].shapes);
    for (const CrtSlab& s : g.host)
        if (crt_slab_kernel_class(s.shapes) != c) return 0;
    return c;
}

hc_status crt_group_run(hc_context ctx, CrtGroup& g) {
    size_t tile = 0;
    for (const CrtSlab& s : g.host) tile = std::max(tile, crt_tile_words(s, g.launch.logv));
    const bool generic = crt_generic(g.host);
    return launch_crt_batch(ctx, g.dev.as<CrtSlab>(), (int)g.host.size(), g.counter.as<int>(), tile, g.tw_words,
                            g.launch, generic, generic ? 0 : crt_group_kernel_class(g));
}

/// Times every launch shape of the candidate set on a scratch copy of a sample of the group's
/// slabs and keeps the fastest.
hc_status crt_group_tune(hc_context ctx, CrtGroup& g, int reps) {
    cudaStream_t st = stream_of(ctx);
    // a sample of at most 4096 slabs, every k-th, each given its own rows in a scratch buffer
    // (the operands stay the batch's own, they are only read); a sample of a few slabs per
    // persistent CTA, so that the last round's imbalance weighs as it will in the batch
    const size_t k = (g.host.size() + 4095) / 4096;
    std::vector<CrtSlab> sample;
    size_t words = 0;
    for (size_t i = 0; i < g.host.size(); i += k) {
        sample.push_back(g.host[i]);
        words += (size_t)g.host[i].dl * g.host[i].dk;
    }
    DBuf scratch(ctx, words * 8);
    CK(cuda_check(cudaMemsetAsync(scratch.p, 0, words * 8, st), "tuning scratch"));
    size_t off = 0;
    for (CrtSlab& s : sample) {
        s.data = scratch.as<int64_t>() + off;
        s.s2 = s.dk;
        off += (size_t)s.dl * s.dk;
    }
    DBuf sdev(ctx, sample.data(), sample.size() * sizeof(CrtSlab));
    DBuf cnt(ctx, sizeof(int));
    cudaEvent_t e0, e1;
    CK(cuda_check(cudaEventCreate(&e0), "tuning event"));
    CK(cuda_check(cudaEventCreate(&e1), "tuning event"));
    CrtLaunch best = g.launch;
    float best_ms = -1;
    const bool generic = crt_generic(g.host);
    const int cls = generic ? 0 : crt_group_kernel_class(g);
    // 128 or 256 threads at 1..4 CTAs per SM
    const CrtLaunch shapes[] = {{128, 1, 0}, {128, 2, 0}, {128, 3, 0}, {128, 4, 0},
                                {256, 1, 0}, {256, 2, 0}, {256, 3, 0}, {256, 4, 0}};
    const int logvs[] = {4, 5, 6};
    hc_status rc = HC_OK;
    for (const CrtLaunch& sh : shapes)
        for (int lv : logvs) {
            CrtLaunch L{sh.threads, sh.ctas_per_sm, lv};
            size_t tile = 0;
            for (const CrtSlab& s : sample) tile = std::max(tile, crt_tile_words(s, lv));
            rc = launch_crt_batch(ctx, sdev.as<CrtSlab>(), (int)sample.size(), cnt.as<int>(), tile, g.tw_words, L,
                                  generic, cls);
            if (rc == HC_ERR_UNSUPPORTED) {  // shape does not fit an SM
                rc = HC_OK;
                continue;
            }
            if (rc) break;
            cudaEventRecord(e0, st);
            for (int r = 0; r < reps && !rc; r++)
                rc = launch_crt_batch(ctx, sdev.as<CrtSlab>(), (int)sample.size(), cnt.as<int>(), tile, g.tw_words,
                                      L, generic, cls);
            if (rc) break;
            cudaEventRecord(e1, st);
            rc = cuda_check(cudaEventSynchronize(e1), "tuning run");
            if (rc) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (best_ms < 0 || ms < best_ms) best_ms = ms, best = L;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    CK(rc);
    CK(cuda_check(cudaStreamSynchronize(st), "tuning"));
    g.launch = best;
    std::lock_guard<std::mutex> lock(crt_tune_mu);
    crt_tuned[g.signature] = best;
    return HC_OK;
}

}  // namespace

extern "C" {

hc_status hc_crt_batch_create(hc_context ctx, const hc_crt_item* items, size_t n, int ops, hc_crt_batch* out) {
    return guard([&] {
        REQUIRE(ctx && out && (items || n == 0), HC_ERR_ARG, "null argument");
        const bool one_launch = ops & HC_CRT_ONE_LAUNCH;
        ops &= ~HC_CRT_ONE_LAUNCH;
        REQUIRE(ops > 0 && ops <= (HC_CRT_FORWARD | HC_CRT_MUL | HC_CRT_INVERSE), HC_ERR_ARG,
                "batched transform: ops must combine HC_CRT_FORWARD, HC_CRT_MUL, HC_CRT_INVERSE");
        auto b = std::make_unique<hc_crt_batch_s>();
        b->ctx = ctx;
        std::vector<CrtSlab> slabs;
        std::vector<size_t> tws;  // staged twiddle words of each slab's two plans
        for (size_t it = 0; it < n; it++) {
            const hc_crt_item& I = items[it];
            hc_ring R = I.ring;
            REQUIRE(R && R->ctx == ctx, HC_ERR_ARG, "batched transform: item ring missing or of another context");
            Base base = base_of(I.base, I.r);
            const int64_t count = I.data.shape[0], r = (int64_t)I.r;
            check_view(I.data, count, r, R->dl(), R->dk(), "batched transform data");
            const bool mul = ops & HC_CRT_MUL;
            if (mul) {
                REQUIRE(I.op.shape[0] == count || I.op.shape[0] == 1, HC_ERR_SHAPE,
                        "batched transform operand: one element per data element, or one for all");
                check_view(I.op, I.op.shape[0], r, R->dl(), R->dk(), "batched transform operand");
            }
            if (count == 0 || r == 0) continue;
            TransformCache& tc = R->transform_cache(base);
            for (int64_t i = 0; i < count; i++)
                for (int64_t j = 0; j < r; j++) {
                    CrtSlab s;
                    std::memset(&s, 0, sizeof(s));
                    s.plan2 = plan_device(tc.plp[j]);
                    s.plan3 = plan_device(tc.pk[j]);
                    s.data = (int64_t*)I.data.ptr + i * I.data.strides[0] + j * I.data.strides[1];
                    s.s2 = I.data.strides[2];
                    if (mul) {
                        s.op = (const int64_t*)I.op.ptr + (I.op.shape[0] == 1 ? 0 : i) * I.op.strides[0] +
                               j * I.op.strides[1];
                        s.op_s2 = I.op.strides[2];
                    }
                    s.kl = (const int64_t*)tc.kl.view().ptr + j * R->dl();
                    s.kk = (const int64_t*)tc.kk.view().ptr + j * R->dk();
                    s.ikl = (const int64_t*)tc.ikl.view().ptr + j * R->dl();
                    s.ikk = (const int64_t*)tc.ikk.view().ptr + j * R->dk();
                    s.n = tc.mods[j].n, s.ninv = tc.mods[j].neg_inv_n;
                    s.dl = (int32_t)R->dl(), s.dk = (int32_t)R->dk();
                    s.ops = ops;
                    {
                        // plan_shape: shape in bits 0..7, fixed schedule in bit 8
                        const int32_t s3 = plan_shape(tc.pk[j]), s2 = plan_shape(tc.plp[j]);
                        s.shapes = (s3 & 0xff) | ((s2 & 0xff) << 8) | (((s3 >> 8) & 1) << 16) | (((s2 >> 8) & 1) << 17);
                    }
                    slabs.push_back(s);
                    tws.push_back(2 * (size_t)(plan_ntw(tc.plp[j]) + plan_ntw(tc.pk[j])));
                }
        }
        REQUIRE(slabs.size() < (size_t)INT32_MAX, HC_ERR_UNSUPPORTED, "batched transform: too many slabs");
        std::map<int, size_t> index;  // shape class -> group
        for (size_t i = 0; i < slabs.size(); i++) {
            const int cls = one_launch ? 0 : crt_slab_class(slabs[i]);
            auto it = index.find(cls);
            if (it == index.end()) {
                it = index.emplace(cls, b->groups.size()).first;
                b->groups.emplace_back();
            }
            CrtGroup& g = b->groups[it->second];
            g.host.push_back(slabs[i]);
            g.tw_words = std::max(g.tw_words, tws[i]);
            g.residues += (int64_t)slabs[i].dl * slabs[i].dk;
        }
        // the group with the most residues first: its launch shape is the batch's reported one
        std::stable_sort(b->groups.begin(), b->groups.end(),
                         [](const CrtGroup& x, const CrtGroup& y) { return x.residues > y.residues; });
        for (CrtGroup& g : b->groups) {
            // largest slabs first: the persistent CTAs finish on the small ones
            std::stable_sort(g.host.begin(), g.host.end(), [](const CrtSlab& x, const CrtSlab& y) {
                return (int64_t)x.dl * x.dk > (int64_t)y.dl * y.dk;
            });
            g.signature = "c" + std::to_string(crt_slab_class(g.host[0])) + ":" + crt_signature(g.host);
            {
                std::lock_guard<std::mutex> lock(crt_tune_mu);
                auto it = crt_tuned.find(g.signature);
                if (it != crt_tuned.end()) g.launch = it->second;
            }
            g.dev = DBuf(ctx, g.host.data(), g.host.size() * sizeof(CrtSlab));
            g.counter = DBuf(ctx, sizeof(int));
        }
        *out = b.release();
    });
}

hc_status hc_crt_batch_run(hc_crt_batch b) {
    return guard([&] {
        REQUIRE(b, HC_ERR_ARG, "null batch");
        for (CrtGroup& g : b->groups) CK(crt_group_run(b->ctx, g));
    });
}

hc_status hc_crt_batch_set_launch(hc_crt_batch b, const hc_crt_launch* l) {
    return guard([&] {
        REQUIRE(b && l, HC_ERR_ARG, "null argument");
        REQUIRE(l->threads >= 32 && l->threads <= 256 && l->threads % 32 == 0, HC_ERR_ARG, "threads per CTA");
        REQUIRE(l->ctas_per_sm >= 1 && l->logv >= 0 && l->logv <= 6, HC_ERR_ARG, "launch shape");
        for (CrtGroup& g : b->groups) g.launch = CrtLaunch{l->threads, l->ctas_per_sm, l->logv};
    });
}

hc_status hc_crt_batch_get_launch(hc_crt_batch b, hc_crt_launch* out) {
    return guard([&] {
        REQUIRE(b && out, HC_ERR_ARG, "null argument");
        const CrtLaunch L = b->groups.empty() ? CrtLaunch{256, 3, 6} : b->groups[0].launch;
        out->threads = L.threads, out->ctas_per_sm = L.ctas_per_sm, out->logv = L.logv;
    });
}

size_t hc_crt_batch_num_slabs(hc_crt_batch b) {
    size_t n = 0;
    if (b)
        for (const CrtGroup& g : b->groups) n += g.host.size();
    return n;
}

hc_status hc_crt_batch_tune(hc_crt_batch b, int reps, hc_crt_launch* chosen) {
    return guard([&] {
        REQUIRE(b, HC_ERR_ARG, "null batch");
        if (reps < 1) reps = 1;
        for (CrtGroup& g : b->groups) CK(crt_group_tune(b->ctx, g, reps));
        if (chosen) CK(hc_crt_batch_get_launch(b, chosen));
    });
}

hc_status hc_crt_batch_destroy(hc_crt_batch b) {
    delete b;
    return HC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------- Galois keysets

/// Galois keys of one gadget split, resident in HBM up to a byte budget; the rest is kept in
/// pinned host memory and staged into two alternating device slots right before use, the copy
/// of the next key running on a copy stream while the current key switch computes.
struct hc_keyset_s {
    hc_ring R = nullptr;
    hc_context ctx = nullptr;  // the ring's context: a keyset may be destroyed after its ring
    Digits digits;
    size_t r_key = 0, key_words = 0, budget = 0, resident_bytes = 0;
    struct Entry {
        DBuf dev;
        void* host = nullptr;
    };
    std::map<uint64_t, Entry> keys;
    DBuf slot[2];
    cudaEvent_t ready[2] = {nullptr, nullptr}, freed[2] = {nullptr, nullptr};
    cudaStream_t copy = nullptr;
    int next_slot = 0;
    uint64_t streamed_keys = 0, streamed_bytes = 0;
    ~hc_keyset_s() {
        for (auto& kv : keys)
            if (kv.second.host) cudaFreeHost(kv.second.host);
        for (int i = 0; i < 2; i++) {
            if (ready[i]) cudaEventDestroy(ready[i]);
            if (freed[i]) cudaEventDestroy(freed[i]);
        }
        if (copy) cudaStreamDestroy(copy);
    }
    size_t key_bytes() const { return key_words * 8; }
    hc_view view_of(void* p) const {
        hc_view v;
        v.ptr = p;
        v.shape[0] = 2 * (int64_t)digits.size(), v.shape[1] = (int64_t)r_key, v.shape[2] = R->dl(), v.shape[3] = R->dk();
        v.strides[3] = 1, v.strides[2] = R->dk(), v.strides[1] = R->dl() * R->dk(), v.strides[0] = (int64_t)r_key * v.strides[1];
        return v;
    }
    /// Issues the copy of a streamed key into the next slot (after that slot's last use).
    int stage(const Entry& e) {
        const int s = next_slot;
        next_slot ^= 1;
        cudaStream_t st = stream_of(R->ctx);
        if (!slot[s].p) slot[s] = DBuf(R->ctx, key_bytes());
        CK(cuda_check(cudaStreamWaitEvent(copy, freed[s], 0), "keyset copy wait"));
        CK(cuda_check(cudaMemcpyAsync(slot[s].p, e.host, key_bytes(), cudaMemcpyHostToDevice, copy), "key stream copy"));
        CK(cuda_check(cudaEventRecord(ready[s], copy), "keyset copy event"));
        (void)st;
        streamed_keys++;
        streamed_bytes += key_bytes();
        return s;
    }
    /// Runs fn(i, key view) for the keys of gs in order on the context stream; resident keys are
    /// used in place, streamed keys are staged one ahead.
    template <typename F>
    void each(const std::vector<uint64_t>& gs, F fn) {
        cudaStream_t st = stream_of(R->ctx);
        std::vector<const Entry*> es;
        for (uint64_t g : gs) {
            auto it = keys.find(g);
            REQUIRE(it != keys.end(), HC_ERR_ARG, "keyset: no Galois key for automorphism " + std::to_string(g));
            es.push_back(&it->second);
        }
        std::vector<int> slot_of(gs.size(), -1);
        size_t pre = 0;  // next key whose copy is not yet issued
        auto issue_next = [&](size_t from) {
            for (pre = std::max(pre, from); pre < es.size(); pre++)
                if (es[pre]->host) {
                    slot_of[pre] = stage(*es[pre]);
                    pre++;
                    return;
                }
        };
        issue_next(0);
        for (size_t i = 0; i < es.size(); i++) {
            hc_view kv;
            if (es[i]->host) {
                const int s = slot_of[i];
                CK(cuda_check(cudaStreamWaitEvent(st, ready[s], 0), "keyset ready wait"));
                issue_next(i + 1);  // overlaps the key switch of key i
                kv = view_of(slot[s].p);
                fn(i, kv);
                CK(cuda_check(cudaEventRecord(freed[s], st), "keyset slot event"));
            } else {
                kv = view_of(es[i]->dev.p);
                fn(i, kv);
            }
        }
    }
};

namespace {

/// bfv_hom_gal (src/bfv.rs:783-841) with the keys of a keyset and one output view per automorphism.
/// bfv_hom_gal (src/bfv.rs:783-841) of B ciphertexts at once (ct [2B, r], rows 2i, 2i + 1; each
/// out [2B, r]) under the automorphisms gs with keys from a keyset: one gadget decomposition of all
/// B ciphertexts, hoisted over gs, and one key-switch launch per automorphism for the whole batch.
void hom_gal_keyset(hc_ring R, const hc_view& ct, const Base& b, const std::vector<uint64_t>& gs, hc_keyset ks,
                    const std::vector<hc_view>& outs) {
    if (gs.empty()) return;
    const int64_t rr = (int64_t)b.size(), B = ct.shape[0] / 2;
    REQUIRE(B >= 1 && ct.shape[0] == 2 * B, HC_ERR_SHAPE, "ciphertexts must have 2 rows each");
    for (auto& o : outs) REQUIRE(o.shape[0] == 2 * B, HC_ERR_SHAPE, "one output row pair per ciphertext");
    Digits dg = clip(ks->digits, b.size());
    REQUIRE(ks->r_key >= b.size(), HC_ERR_SHAPE, "keyset keys cover fewer RNS factors than the ciphertext");
    for (uint64_t g : gs)  // refused before any work is queued
        REQUIRE(ks->keys.count(g), HC_ERR_ARG, "keyset: no Galois key for automorphism " + std::to_string(g));
    Tensor c1(R->ctx, B, rr, R->dl(), R->dk());
    const hc_view c1_crt = vstep(ct, 1, 2, B);
    R->transform(c1.view(), b, true, nullptr, &c1_crt);
    Tensor parts = gadget_decompose(R, c1.view(), b, dg);
    hc_view c0 = vstep(ct, 0, 2, B);
    // consecutive key switches over the same digits alternate their tile order (KsArgs::reverse)
    size_t launched = 0;
    ks->each(gs, [&](size_t gi, const hc_view& key) {
        PermCache& pc = R->perms(gs[gi]);
        keyswitch(R, parts.view(), key, b, dg.size(), &c0, nullptr, outs[gi], pc.p2.as<uint32_t>(), pc.p3.as<uint32_t>(),
                  (launched++ & 1) != 0);
    });
}

/// src/dbfv.rs:97-121
std::vector<std::vector<i128>> balanced_digits_vec(std::vector<i128> cur, i128 b, size_t max_digits) {
    std::vector<std::vector<i128>> out;
    for (size_t it = 0; it < max_digits; it++) {
        bool zero = true;
        for (i128 v : cur) zero = zero && v == 0;
        if (zero) break;
        std::vector<i128> rems;
        for (i128& v : cur) {
            i128 rem = v % b;  // cmod: the representative in (-b/2, b/2] (src/ring.rs:94-104)
            if (rem < 0) rem += b;
            if (rem > b / 2) rem -= b;
            rems.push_back(rem);
            v = (v - rem) / b;
        }
        out.push_back(rems);
    }
    return out;
}

/// src/bootstrap/homcrt.rs:335-339
std::pair<size_t, size_t> bsgs_split(size_t len) {
    size_t best = 1, best_cost = (size_t)-1;
    for (size_t count = 1; count <= len; count++) {
        size_t cost = count + 3 * ((len - 1) / count + 1);  // UNHOISTED_OVERHEAD = 3 (homcrt.rs:333)
        if (cost < best_cost) best_cost = cost, best = count;
    }
    return {best, (len - 1) / best + 1};
}

uint64_t pow_mod_m(uint64_t g, size_t e, uint64_t m) {
    uint64_t r = 1;
    for (size_t i = 0; i < e; i++) r = (uint64_t)((u128)r * g % m);
    return r;
}

}  // namespace

extern "C" {

hc_status hc_keyset_create(hc_ring R, const size_t* digits, size_t d, size_t r_key, size_t hbm_budget_bytes,
                           hc_keyset* out) {
    return guard([&] {
        REQUIRE(R && out, HC_ERR_ARG, "null argument");
        REQUIRE(d > 0 && r_key > 0, HC_ERR_ARG, "keyset: digits and key RNS length");
        auto ks = std::make_unique<hc_keyset_s>();
        ks->R = R;
        ks->ctx = R->ctx;
        ks->digits = digits_of(digits, d);
        ks->r_key = r_key;
        ks->key_words = 2 * d * r_key * (size_t)R->dl() * (size_t)R->dk();
        ks->budget = hbm_budget_bytes;
        CK(cuda_check(cudaStreamCreateWithFlags(&ks->copy, cudaStreamNonBlocking), "keyset copy stream"));
        for (int i = 0; i < 2; i++) {
            CK(cuda_check(cudaEventCreateWithFlags(&ks->ready[i], cudaEventDisableTiming), "keyset event"));
            CK(cuda_check(cudaEventCreateWithFlags(&ks->freed[i], cudaEventDisableTiming), "keyset event"));
            CK(cuda_check(cudaEventRecord(ks->freed[i], stream_of(R->ctx)), "keyset event"));
        }
        *out = ks.release();
    });
}

hc_status hc_keyset_add(hc_keyset ks, uint64_t g, hc_view key) {
    return guard([&] {
        REQUIRE(ks, HC_ERR_ARG, "null keyset");
        hc_ring R = ks->R;
        check_view(key, 2 * (int64_t)ks->digits.size(), (int64_t)ks->r_key, R->dl(), R->dk(), "Galois key");
        REQUIRE(key.strides[2] == R->dk() && key.strides[1] == R->dl() * R->dk() &&
                    key.strides[0] == (int64_t)ks->r_key * R->dl() * R->dk(),
                HC_ERR_SHAPE, "Galois key must be contiguous");
        REQUIRE(!ks->keys.count(g), HC_ERR_ARG, "keyset: automorphism already has a key");
        hc_keyset_s::Entry e;
        cudaStream_t st = stream_of(R->ctx);
        if (ks->resident_bytes + ks->key_bytes() <= ks->budget) {
            e.dev = DBuf(R->ctx, ks->key_bytes());
            CK(cuda_check(cudaMemcpyAsync(e.dev.p, key.ptr, ks->key_bytes(), cudaMemcpyDeviceToDevice, st), "key copy"));
            ks->resident_bytes += ks->key_bytes();
        } else {
            count_alloc();
            CK(cuda_check(cudaMallocHost(&e.host, ks->key_bytes()), "pinned key allocation"));
            CK(cuda_check(cudaMemcpyAsync(e.host, key.ptr, ks->key_bytes(), cudaMemcpyDeviceToHost, st), "key copy"));
            CK(cuda_check(cudaStreamSynchronize(st), "key copy"));
        }
        ks->keys[g] = std::move(e);
    });
}

hc_status hc_keyset_stats(hc_keyset ks, size_t* resident, size_t* streamed, uint64_t* streamed_keys,
                          uint64_t* streamed_bytes) {
    return guard([&] {
        REQUIRE(ks, HC_ERR_ARG, "null keyset");
        size_t res = 0, str = 0;
        for (auto& kv : ks->keys) (kv.second.host ? str : res)++;
        if (resident) *resident = res;
        if (streamed) *streamed = str;
        if (streamed_keys) *streamed_keys = ks->streamed_keys;
        if (streamed_bytes) *streamed_bytes = ks->streamed_bytes;
    });
}

hc_status hc_keyset_destroy(hc_keyset ks) {
    if (ks) cudaStreamSynchronize(stream_of(ks->ctx));
    delete ks;
    return HC_OK;
}

hc_status hc_bfv_hom_gal_keyset(hc_ring R, hc_view ct, const size_t* base, size_t r, const uint64_t* gs, size_t ngs,
                                hc_keyset ks, hc_view out) {
    return guard([&] {
        REQUIRE(R && ks, HC_ERR_ARG, "null argument");
        if (ngs == 0) return;
        REQUIRE(gs, HC_ERR_ARG, "null automorphism list");
        Base b = base_of(base, r);
        check_view(ct, 2, (int64_t)r, R->dl(), R->dk(), "ciphertext");
        check_view(out, 2 * (int64_t)ngs, (int64_t)r, R->dl(), R->dk(), "output");
        std::vector<hc_view> outs;
        for (size_t i = 0; i < ngs; i++) outs.push_back(vrows(out, 2 * (int64_t)i, 2 * (int64_t)i + 2));
        hom_gal_keyset(R, ct, b, std::vector<uint64_t>(gs, gs + ngs), ks, outs);
    });
}

hc_status hc_bfv_hom_gal_batch_keyset(hc_ring R, hc_view ct, const size_t* base, size_t r, uint64_t g, hc_keyset ks,
                                      hc_view out) {
    return guard([&] {
        REQUIRE(R && ks, HC_ERR_ARG, "null argument");
        Base b = base_of(base, r);
        REQUIRE(ct.shape[0] >= 2 && ct.shape[0] % 2 == 0, HC_ERR_SHAPE, "ciphertexts must have 2 rows each");
        check_view(ct, ct.shape[0], (int64_t)r, R->dl(), R->dk(), "ciphertexts");
        check_view(out, ct.shape[0], (int64_t)r, R->dl(), R->dk(), "output");
        hom_gal_keyset(R, ct, b, std::vector<uint64_t>{g}, ks, std::vector<hc_view>{out});
    });
}

hc_status hc_dbfv_hom_cyclic_transform(hc_ring R, size_t log2_b, size_t log2_t, uint64_t g, const int64_t* coeffs,
                                       size_t len, hc_view ct, const size_t* base, size_t r, hc_keyset ks, hc_view out,
                                       size_t* out_rows) {
    return guard([&] {
        REQUIRE(R && ks && out_rows, HC_ERR_ARG, "null argument");
        REQUIRE(log2_b >= 1 && log2_t >= 1 && log2_t <= 126, HC_ERR_ARG, "t = 2^log2_t must be between 2 and 2^126");
        REQUIRE(len == 0 || coeffs, HC_ERR_ARG, "null coefficients");
        const size_t digits = (log2_t - 1) / log2_b + 1;
        REQUIRE(log2_b <= 125, HC_ERR_ARG, "digit base too large");
        const i128 bb = (i128)1 << log2_b;
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r, dl = R->dl(), dk = R->dk();
        REQUIRE(ct.shape[0] % 2 == 0, HC_ERR_SHAPE, "dBFV ciphertext rows");
        const size_t d = (size_t)ct.shape[0] / 2;
        REQUIRE(d <= digits, HC_ERR_SHAPE, "ciphertext has more digits than the modulus");
        check_view(ct, ct.shape[0], rr, dl, dk, "dBFV ciphertext");
        check_view(out, 2 * (int64_t)digits, rr, dl, dk, "output");
        *out_rows = 0;
        if (len == 0) return;
        // the L' coefficients' balanced digits as CRT-basis tensors [1, r, deg_L', 1]
        // (src/ring.rs:1227-1250), all in one batch
        std::vector<std::vector<std::vector<i128>>> bd(len);
        std::vector<size_t> first(len, 0);
        size_t nt = 0;
        for (size_t i = 0; i < len; i++) {
            std::vector<i128> c((size_t)dl);
            for (int64_t k = 0; k < dl; k++) {
                const int64_t* w = coeffs + 2 * (i * (size_t)dl + (size_t)k);
                c[(size_t)k] = (i128)(((u128)(uint64_t)w[1] << 64) | (uint64_t)w[0]);
            }
            bd[i] = balanced_digits_vec(c, bb, digits);
            first[i] = nt;
            nt += bd[i].size();
        }
        Tensor L;
        if (nt > 0) {
            L = Tensor(R->ctx, (int64_t)nt, rr, dl, 1);
            std::vector<int64_t> vals;
            for (size_t i = 0; i < len; i++)
                for (auto& cv : bd[i])
                    for (size_t idx : b) {
                        const int64_t p = R->prime(idx);
                        for (i128 cf : cv) vals.push_back(mont_repr((int64_t)(cf % (i128)p), p));
                    }
            R->upload_async(L.view().ptr, vals.data(), vals.size());
            TransformCache& tc = R->transform_cache(b);
            CK(hc_ntt_mul_mont64_dim(R->ctx, L.view(), tc.plp.data(), r, HC_DIM2, tc.kl.view(), tc.mods.data(), r));
            CK(hc_intt_mont64_dim(R->ctx, L.view(), tc.plp.data(), r, HC_DIM2));
        }
        auto ltensor = [&](size_t i, size_t jj) { return vrows(L.view(), (int64_t)(first[i] + jj), (int64_t)(first[i] + jj + 1)); };
        // a dBFV batch O of `od` digits in CRT basis, reduced from a fresh accumulator
        Tensor O;
        size_t od = 0;
        auto finish = [&](Wide& acc, size_t used) {
            Tensor n(R->ctx, 2 * (int64_t)used, rr, dl, dk, false, false);
            if (used > 0) acc.reduce_rows_into(n.view(), 2 * used);
            O = std::move(n);
            od = used;
        };
        if (len == 1) {
            // dbfv_hom_fma_element_lprime with an empty summand (src/dbfv.rs:431-453)
            if (d == 0 || bd[0].empty()) return;
            Wide acc(R, 2 * (int64_t)digits, b);
            const size_t nd = std::min(digits, d + bd[0].size() - 1);
            for (size_t i = 0; i < d; i++)
                for (size_t j = 0; j < bd[0].size(); j++)
                    if (i + j < nd)
                        acc.fma(2 * (i + j), 2 * (i + j) + 2, vrows(ct, 2 * (int64_t)i, 2 * (int64_t)i + 2), 1,
                                ltensor(0, j), 1);
            finish(acc, nd);
        } else {
            const auto sp = bsgs_split(len);
            const size_t baby = sp.first, giant_steps = sp.second;
            const uint64_t m = R->field.m();
            std::vector<uint64_t> baby_exps;
            for (size_t j = 1; j < baby; j++) baby_exps.push_back(pow_mod_m(g, j, m));
            // babys: block j (rows j 2d .. (j + 1) 2d) = sigma^j(ct)
            Tensor B(R->ctx, (int64_t)(baby * 2 * d), rr, dl, dk, false, false);
            if (d > 0) {
                // all d digits in one hoisted batch: block j holds sigma^j of every digit
                CK(hc_assign(R->ctx, vrows(B.view(), 0, 2 * (int64_t)d), ct));
                std::vector<hc_view> outs;
                for (size_t j = 1; j < baby; j++)
                    outs.push_back(vrows(B.view(), (int64_t)(j * 2 * d), (int64_t)((j + 1) * 2 * d)));
                hom_gal_keyset(R, vrows(B.view(), 0, 2 * (int64_t)d), b, baby_exps, ks, outs);
            }
            const uint64_t giant_exp = pow_mod_m(g, baby, m);
            for (size_t giant = giant_steps; giant-- > 0;) {
                if (giant != giant_steps - 1 && od > 0) {
                    Tensor rot(R->ctx, 2 * (int64_t)od, rr, dl, dk, false, false);
                    hom_gal_keyset(R, O.view(), b, {giant_exp}, ks, {rot.view()});  // all od digits at once
                    O = std::move(rot);
                }
                const size_t nterm = std::min(baby, len - giant * baby);
                size_t max_new = 0;
                for (size_t j = 0; j < nterm; j++) {
                    const size_t nr = bd[giant * baby + j].size();
                    if (d > 0 && nr > 0) max_new = std::max(max_new, std::min(digits, d + nr - 1));
                }
                // one fused launch per output digit: the inner product over the convolution
                // diagonal (src/dbfv.rs:291-352), the carried digit through mont(1) and the
                // reduction the accumulator's bound asks for (src/ring.rs:365, :846-865)
                const size_t used = std::max(max_new, od);
                Tensor n(R->ctx, 2 * (int64_t)used, rr, dl, dk, false, false);
                const u128 mp2 = (u128)R->max_p(b) * (u128)R->max_p(b);
                const int64_t minp = R->min_p(b);
                const KMods km = R->kmods(b);
                const int64_t* one = R->one_dev(b);
                std::vector<int> lf(nterm, 0), lc(nterm, 0);
                for (size_t j = 0; j < nterm; j++) {
                    lf[j] = (int)first[giant * baby + j];
                    lc[j] = (int)bd[giant * baby + j].size();
                }
                std::vector<unsigned char> fullv(used);
                for (size_t k = 0; k < used; k++) {
                    size_t cnt = 0;  // the inner product's terms for output digit k
                    for (size_t j = 0; j < nterm && d > 0; j++)
                        for (size_t jj = 0; jj < (size_t)lc[j] && jj <= k; jj++)
                            if (k - jj < d) cnt++;
                    fullv[k] = needs_full((u128)cnt * mp2 + (k < od ? mp2 : 0), minp);
                }
                KView addv = od > 0 ? kv(O.view()) : KView();
                CK(launch_giant(R->ctx, kv(B.view()), nt > 0 ? kv(L.view()) : KView(), d > 0 ? (int)nterm : 0, (int)d,
                                lf.data(), lc.data(), od > 0 ? &addv : nullptr, (int)od, fullv.data(), (int)used,
                                kv(n.view()), km, one));
                O = std::move(n);
                od = used;
            }
        }
        if (od > 0) CK(hc_assign(R->ctx, vrows(out, 0, 2 * (int64_t)od), O.view()));
        *out_rows = 2 * od;
    });
}

}  // extern "C"

// ------------------------------------------------------------------------- dBFV reduction path
// split_overflow, dbfv_reduce, dbfv_enc, dbfv_mul_convolve / dbfv_hom_mul (src/dbfv.rs:661-1143).
// The big-integer constants are evaluated modulo 2^128 (wrapping products of the primes) and
// modulo each prime.

namespace {

/// src/dbfv.rs:762-768
i128 inv_mod_2_128(i128 q) {
    u128 x = (u128)q, qq = (u128)q;
    for (int i = 0; i < 6; i++) x = x * (2 - qq * x);
    return (i128)x;
}

u128 q_mod_2_128(hc_ring R, const Base& b) {
    u128 q = 1;
    for (size_t i : b) q *= (u128)R->prime(i);
    return q;
}

/// round(Q / 2^k) modulo p (Q odd: no ties)
std::function<int64_t(int64_t)> delta_pow2(hc_ring R, const Base& b, size_t k) {
    const u128 c = q_mod_2_128(R, b) & (((u128)1 << k) - 1);
    const int64_t extra = c >= ((u128)1 << (k - 1)) ? 1 : 0;
    return [c, k, extra](int64_t p) {
        int64_t cp = (int64_t)(c % (u128)p), two = 1;
        for (size_t i = 0; i < k; i++) two = mulm(two, 2, p);
        return emod(mulm(emod(-cp, p), invm(two, p), p) + extra, p);
    };
}

int64_t pow2_mod(size_t e, int64_t p) {
    int64_t v = 1;
    for (size_t i = 0; i < e; i++) v = mulm(v, 2, p);
    return v;
}

/// [1, r, 1, 1] tensor of mont(mont(smallest lift)) (src/ring.rs:907-920)
Tensor scalar_tensor_big_mont2(hc_ring R, const Base& b, const std::function<int64_t(int64_t)>& res) {
    std::vector<int64_t> v;
    for (size_t i : b) {
        const int64_t p = R->prime(i);
        v.push_back(mont_repr(mont_repr(centred(res(p), p), p), p));
    }
    Tensor t(R->ctx, 1, (int64_t)b.size(), 1, 1);
    CK(hc_import(R->ctx, t.view(), v.data(), v.size()));
    return t;
}

/// rows [s, e) of dimension 1
hc_view dim1(hc_view v, int64_t s, int64_t e) {
    v.ptr = (char*)v.ptr + s * v.strides[1] * 8;
    v.shape[1] = e - s;
    return v;
}

/// SplitOverflowData (src/dbfv.rs:735-849)
struct SplitData {
    size_t log2_r = 0, log2_gamma = 0;
    i128 q_mod_r = 0, neg_q_inv_mod_r = 0;
    Tensor rqinv, matrix;
    std::vector<Tensor> neg_b_delta_mont2;
    size_t limbs() const { return log2_r <= 62 ? 1 : 2; }
    SplitData(hc_ring R, size_t log2_b, size_t log2_t, const Base& b) {
        log2_r = log2_t - log2_b;
        REQUIRE(log2_r >= 1 && log2_r <= 126, HC_ERR_ARG, "t/b must be between 2 and 2^126");
        const size_t L = limbs();
        const u128 rmask = ((u128)1 << log2_r) - 1;
        const int64_t mx = R->max_p(b), mn = R->min_p(b);
        log2_gamma = std::max<size_t>(64, bitlen_u128(4 * (u128)b.size() * (u128)mx + 1));
        REQUIRE(log2_gamma <= 126, HC_ERR_UNSUPPORTED, "split overflow precision");
        const i128 gamma = (i128)1 << log2_gamma;
        REQUIRE((gamma / mn + 1) <= I128MAX / ((i128)mx * (i128)b.size()), HC_ERR_ARG, "split overflow matrix range");
        std::vector<i128> qpr;
        for (size_t i : b) {
            u128 q = 1;
            for (size_t j : b)
                if (j != i) q *= (u128)R->prime(j);
            qpr.push_back((i128)(q & rmask));
        }
        std::vector<int64_t> mat;
        for (i128 c : qpr) mat.push_back((int64_t)c);  // split_i128_limbs(c).0 (src/hal/mod.rs:71-76)
        if (L == 2)
            for (i128 c : qpr) mat.push_back((int64_t)((c - (i128)(int64_t)c) >> 64));
        for (size_t i : b) {
            const i128 p = R->prime(i);
            mat.push_back((int64_t)((gamma + p / 2) / p));
        }
        matrix = Tensor(R->ctx, 1, (int64_t)L + 1, (int64_t)b.size(), 1);
        CK(hc_import(R->ctx, matrix.view(), mat.data(), mat.size()));
        q_mod_r = (i128)(q_mod_2_128(R, b) & rmask);
        neg_q_inv_mod_r = (i128)((u128)(-inv_mod_2_128(q_mod_r)) & rmask);
        // smallest lifts of R (Q/p)^-1 mod p (src/ring.rs:1029-1043)
        std::vector<int64_t> qv;
        for (size_t i : b) {
            const int64_t p = R->prime(i);
            int64_t qo = 1;
            for (size_t j : b)
                if (j != i) qo = mulm(qo, R->prime(j) % p, p);
            qv.push_back(centred(mulm(invm(qo, p), pow2_mod(log2_r, p), p), p));
        }
        rqinv = Tensor(R->ctx, 1, (int64_t)b.size(), 1, 1);
        CK(hc_import(R->ctx, rqinv.view(), qv.data(), qv.size()));
        auto delta = delta_pow2(R, b, log2_t);
        for (size_t k = 0; k < L; k++)
            neg_b_delta_mont2.push_back(scalar_tensor_big_mont2(R, b, [&](int64_t p) {
                return emod(-mulm(mulm(delta(p), pow2_mod(log2_b, p), p), pow2_mod(64 * k, p), p), p);
            }));
    }
};

/// src/dbfv.rs:891-950: x <- x_lo in place; returns the overflow limbs [count, limbs, ...]
Tensor split_overflow(hc_ring R, const SplitData& D, const hc_view& x, u128 x_bound, const Base& b) {
    const int64_t count = x.shape[0], r = (int64_t)b.size(), L = (int64_t)D.limbs();
    std::vector<hc_modulus> m = R->mods(b);
    Tensor lifts(R->ctx, count, r, R->dl(), R->dk(), false, false);
    CK(hc_assign(R->ctx, lifts.view(), x));
    CK(hc_mul_mont64(R->ctx, lifts.view(), D.rqinv.view(), m.data(), m.size()));
    Tensor sums(R->ctx, count, L + 1, R->dl(), R->dk(), true, false);
    CK(hc_matmul_i64(R->ctx, sums.view(), D.matrix.view(), lifts.view()));
    Tensor overflow(R->ctx, count, L, R->dl(), R->dk(), false, false);
    if (L == 1) {
        CK(hc_bconv_correct_pow2(R->ctx, overflow.view(), sums.view(), (int64_t)D.q_mod_r, (int64_t)D.neg_q_inv_mod_r,
                                 D.log2_gamma, D.log2_r));
    } else {
        const int64_t f0[2] = {(int64_t)(uint64_t)D.q_mod_r, (int64_t)(D.q_mod_r >> 64)};
        const int64_t f1[2] = {(int64_t)(uint64_t)D.neg_q_inv_mod_r, (int64_t)(D.neg_q_inv_mod_r >> 64)};
        CK(hc_bconv_correct_pow2_wide(R->ctx, overflow.view(), sums.view(), f0, f1, D.log2_gamma, D.log2_r));
    }
    Wide acc(R, count, b);
    for (int64_t k = 0; k < L; k++) acc.fma_unbounded(0, (size_t)count, dim1(overflow.view(), k, k + 1), D.neg_b_delta_mont2[(size_t)k].view());
    acc.add(0, (size_t)count, x, x_bound);
    acc.reduce_into(x);
    return overflow;
}

/// The reduction's tables of one (log2 b, log2 t, base): SplitOverflowData and the carries'
/// delta factors, built once per ring (their uploads would otherwise block the host every call).
struct DbfvTables {
    SplitData D;
    std::vector<Tensor> delta_mont2;
    DbfvTables(hc_ring R, size_t log2_b, size_t log2_t, const Base& b) : D(R, log2_b, log2_t, b) {
        auto delta = delta_pow2(R, b, log2_t);
        for (size_t k = 0; k < D.limbs(); k++)
            delta_mont2.push_back(
                scalar_tensor_big_mont2(R, b, [&](int64_t p) { return mulm(delta(p), pow2_mod(64 * k, p), p); }));
    }
};

const DbfvTables& dbfv_tables(hc_ring R, size_t log2_b, size_t log2_t, const Base& b) {
    const auto key = std::make_tuple(log2_b, log2_t, b);
    auto it = R->dbfv_cache.find(key);
    if (it == R->dbfv_cache.end())
        it = R->dbfv_cache.emplace(key, std::make_shared<DbfvTables>(R, log2_b, log2_t, b)).first;
    return *static_cast<const DbfvTables*>(it->second.get());
}

/// src/dbfv.rs:968-1032, period basis in and out; returns the [2 digits, r] result
Tensor dbfv_reduce(hc_ring R, size_t log2_b, size_t log2_t, const hc_view& ct, u128 bound, const Base& b,
                   size_t* rows_out) {
    const size_t digits = (log2_t - 1) / log2_b + 1, d = (size_t)ct.shape[0] / 2;
    REQUIRE(d <= digits, HC_ERR_SHAPE, "ciphertext has more digits than the modulus");
    const int64_t rr = (int64_t)b.size();
    if (digits == 1 || d == 0) {
        Tensor out(R->ctx, 2 * (int64_t)d, rr, R->dl(), R->dk(), false, false);
        if (d) CK(hc_assign(R->ctx, out.view(), ct));
        *rows_out = 2 * d;
        return out;
    }
    const DbfvTables& T = dbfv_tables(R, log2_b, log2_t, b);
    const SplitData& D = T.D;
    const std::vector<Tensor>& delta_mont2 = T.delta_mont2;
    Tensor result(R->ctx, 2 * (int64_t)digits, rr, R->dl(), R->dk());
    CK(hc_assign(R->ctx, vrows(result.view(), 0, 2 * (int64_t)d), ct));
    Tensor carry;
    bool have = false;
    for (size_t i = 0; i < digits; i++) {
        const u128 in_bound = i < d ? bound : 1;
        hc_view rows = vrows(result.view(), 2 * (int64_t)i, 2 * (int64_t)i + 2);
        if (have) {
            Wide acc(R, 2, b);
            for (size_t k = 0; k < delta_mont2.size(); k++)
                acc.fma_unbounded(0, 2, dim1(carry.view(), (int64_t)k, (int64_t)k + 1), delta_mont2[k].view());
            acc.add(0, 2, rows, in_bound);
            acc.reduce_into(rows);
        }
        carry = split_overflow(R, D, rows, have ? 1 : in_bound, b);
        have = true;
    }
    *rows_out = 2 * digits;
    return result;
}

}  // namespace

extern "C" {

hc_status hc_dbfv_reduce(hc_ring R, size_t log2_b, size_t log2_t, hc_view ct, const size_t* base, size_t r,
                         uint64_t bound, hc_view out, size_t* out_rows) {
    return guard([&] {
        REQUIRE(R && out_rows, HC_ERR_ARG, "null argument");
        REQUIRE(log2_b >= 1 && log2_t >= 1 && log2_t <= 126, HC_ERR_ARG, "t = 2^log2_t must be between 2 and 2^126");
        Base b = base_of(base, r);
        REQUIRE(ct.shape[0] % 2 == 0, HC_ERR_SHAPE, "dBFV ciphertext rows");
        check_view(ct, ct.shape[0], (int64_t)r, R->dl(), R->dk(), "dBFV ciphertext");
        size_t rows = 0;
        Tensor res = dbfv_reduce(R, log2_b, log2_t, ct, bound, b, &rows);
        REQUIRE(out.shape[0] >= (int64_t)rows, HC_ERR_SHAPE, "output has too few rows");
        check_view(out, out.shape[0], (int64_t)r, R->dl(), R->dk(), "output");
        if (rows) CK(hc_assign(R->ctx, vrows(out, 0, (int64_t)rows), res.view()));
        *out_rows = rows;
    });
}

hc_status hc_dbfv_enc(hc_ring R, uint64_t* st, size_t log2_b, size_t log2_t, const size_t* base, size_t r,
                      const int64_t* ptxt, hc_view sk, double log2_alpha, hc_view out) {
    return guard([&] {
        REQUIRE(R && st && ptxt, HC_ERR_ARG, "null argument");
        REQUIRE(log2_b >= 1 && log2_t >= 1 && log2_t <= 126, HC_ERR_ARG, "t = 2^log2_t must be between 2 and 2^126");
        const size_t digits = (log2_t - 1) / log2_b + 1;
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r;
        check_view(out, 2 * (int64_t)digits, rr, R->dl(), R->dk(), "dBFV ciphertext");
        const double la = log2_alpha + (double)(log2_b * (digits - 1));  // src/dbfv.rs:602-604
        const i128 t = (i128)1 << log2_t;
        const int64_t tw[2] = {(int64_t)(uint64_t)t, (int64_t)(t >> 64)};
        CK(hc_bfv_enc(R, st, base, r, tw, ptxt, sk, la, vrows(out, 0, 2)));
        if (digits == 1) return;
        for (size_t i = 1; i < digits; i++) enc_zero(R, b, sk, st, la, vrows(out, 2 * (int64_t)i, 2 * (int64_t)i + 2));
        Tensor pb(R->ctx, 2 * (int64_t)digits, rr, R->dl(), R->dk(), false, false);
        CK(hc_assign(R->ctx, pb.view(), out));
        R->transform(pb.view(), b, true);
        size_t rows = 0;
        Tensor red = dbfv_reduce(R, log2_b, log2_t, pb.view(), 1, b, &rows);
        R->transform(red.view(), b, false);
        CK(hc_assign(R->ctx, out, red.view()));
        CK(hc_synchronize(R->ctx));
    });
}

hc_status hc_dbfv_hom_mul(hc_ring R, size_t log2_b, size_t log2_t, hc_view lhs, hc_view rhs, const size_t* base, size_t r,
                          hc_view rk, const size_t* digits, size_t d, int period_output, hc_view out, size_t* out_rows) {
    return guard([&] {
        REQUIRE(R && out_rows, HC_ERR_ARG, "null argument");
        REQUIRE(log2_b >= 1 && log2_t >= 1 && log2_t <= 126, HC_ERR_ARG, "t = 2^log2_t must be between 2 and 2^126");
        const size_t mdig = (log2_t - 1) / log2_b + 1;
        Base b = base_of(base, r);
        const int64_t rr = (int64_t)r;
        REQUIRE(lhs.shape[0] % 2 == 0 && rhs.shape[0] % 2 == 0, HC_ERR_SHAPE, "dBFV ciphertext rows");
        check_view(lhs, lhs.shape[0], rr, R->dl(), R->dk(), "lhs");
        check_view(rhs, rhs.shape[0], rr, R->dl(), R->dk(), "rhs");
        size_t r1 = 0, r2 = 0;
        Tensor l = dbfv_reduce(R, log2_b, log2_t, lhs, 1, b, &r1), rt = dbfv_reduce(R, log2_b, log2_t, rhs, 1, b, &r2);
        *out_rows = 0;
        if (r1 == 0 || r2 == 0) return;
        const size_t d1 = r1 / 2, d2 = r2 / 2, d_out = std::min(mdig, d1 + d2 - 1);
        check_view(out, out.shape[0], rr, R->dl(), R->dk(), "output");
        REQUIRE(out.shape[0] >= 2 * (int64_t)d_out, HC_ERR_SHAPE, "output has too few rows");
        Tensor ll = lift_to_extended(R, vrows(l.view(), 0, (int64_t)r1), nullptr, b);
        Tensor rl = lift_to_extended(R, vrows(rt.view(), 0, (int64_t)r2), nullptr, b);
        Base lifted = b;
        for (int64_t i = rr; i < ll.shape[1]; i++) lifted.push_back(R->initial_len + (size_t)(i - rr));
        // all 3-component digit products, rows 3k .. 3k + 3 for output digit k (src/dbfv.rs:1081-1126)
        Wide acc(R, 3 * (int64_t)d_out, lifted);
        auto row = [](const Tensor& t, size_t i) { return vrows(t.view(), (int64_t)i, (int64_t)i + 1); };
        for (size_t k = 0; k < d_out; k++) {
            std::vector<hc_view> a0, b0, a1, b1, a2, b2;
            const size_t jlo = k >= d2 - 1 ? k - (d2 - 1) : 0, jhi = std::min(k, d1 - 1);
            for (size_t j = jlo; j <= jhi; j++) {
                a0.push_back(row(ll, 2 * j)), b0.push_back(row(rl, 2 * (k - j)));
                a1.push_back(row(ll, 2 * j)), b1.push_back(row(rl, 2 * (k - j) + 1));
                a1.push_back(row(ll, 2 * j + 1)), b1.push_back(row(rl, 2 * (k - j)));
                a2.push_back(row(ll, 2 * j + 1)), b2.push_back(row(rl, 2 * (k - j) + 1));
            }
            acc.inner_product(3 * k, 3 * k + 1, a0, b0);
            acc.inner_product(3 * k + 1, 3 * k + 2, a1, b1);
            acc.inner_product(3 * k + 2, 3 * k + 3, a2, b2);
        }
        Tensor prod(R->ctx, 3 * (int64_t)d_out, (int64_t)lifted.size(), R->dl(), R->dk(), false, false);
        acc.reduce_into(prod.view());
        R->transform(prod.view(), lifted, true);
        const i128 t = (i128)1 << log2_t;
        Tensor resc = rescale_to_base(R, prod.view(), lifted, r, t);
        // relinearisation of every output digit at once (src/bfv.rs:699-741)
        const int64_t D = (int64_t)d_out;
        Digits dg = clip(digits_of(digits, d), r);
        REQUIRE(rk.shape[0] >= 2 * (int64_t)dg.size() && rk.shape[1] >= rr, HC_ERR_SHAPE, "relinearisation key shape");
        Tensor c2(R->ctx, D, rr, R->dl(), R->dk(), false, false);
        CK(hc_assign(R->ctx, c2.view(), vstep(resc.view(), 2, 3, D)));
        Tensor parts = gadget_decompose(R, c2.view(), b, dg);
        hc_view c0 = vstep(resc.view(), 0, 3, D), c1 = vstep(resc.view(), 1, 3, D);
        hc_view o = vrows(out, 0, 2 * D);
        if (!period_output) {
            R->transform(c0, b, false);
            R->transform(c1, b, false);
            keyswitch(R, parts.view(), rk, b, dg.size(), &c0, &c1, o);
        } else {
            keyswitch(R, parts.view(), rk, b, dg.size(), nullptr, nullptr, o);
            R->transform(o, b, true);
            CK(hc_add_i64(R->ctx, vstep(o, 0, 2, D), c0));
            CK(hc_add_i64(R->ctx, vstep(o, 1, 2, D), c1));
        }
        *out_rows = 2 * d_out;
    });
}

}  // extern "C"

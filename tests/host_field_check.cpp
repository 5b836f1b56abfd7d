// Host build of pyzkp_gb300/csrc/host_field.hpp (the library's host-side field code: final
// MSM combination, twiddle and scale tables). Reads records of two 32-byte little-endian
// canonical elements (a, b) from argv[2] for the field named by argv[1] ("fr" or "fq") and
// writes, per record, mul(a, b), inv(a) (zero for a == 0), add(a, b), sub(a, b) and
// to_mont(a) to argv[3]. With argv[1] "g1" a record (k, n) gives the affine canonical
// coordinates of [2^(n mod 48)] P for P = [k mod 2^64] G1 (XYZZ double-and-add, then n XYZZ
// doublings, as in the window combination). With argv[1] "fq2" a record (a0, a1) of
// canonical Fq values gives (a0 + a1 u)^2 in canonical form by csqr and by cmul (u^2 = -1).
// Built and checked by tests/test_host_field.py.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../pyzkp_gb300/csrc/host_field.hpp"

static void put_affine(const zkh::Xyzz& p, FILE* out) {
    zkh::F4 x, y;
    zkh::xyzz_to_affine_canonical(p, &x, &y);
    std::fwrite(x.v, 8, 4, out);
    std::fwrite(y.v, 8, 4, out);
}

static int curve_mode(const std::vector<zkh::F4>& v, FILE* out) {
    const zkh::Field& F = zkh::fq();
    zkh::Xyzz g;
    g.X = zkh::to_mont(F, zkh::F4{{1, 0, 0, 0}});
    g.Y = zkh::to_mont(F, zkh::F4{{2, 0, 0, 0}});
    g.ZZ = zkh::one(F);
    g.ZZZ = zkh::one(F);
    for (size_t i = 0; i < v.size(); i += 2) {
        const uint64_t k = v[i].v[0];
        const uint32_t n = (uint32_t)(v[i + 1].v[0] % 48);
        zkh::Xyzz p = zkh::xyzz_inf();
        for (int b = 63; b >= 0; b--) {
            p = zkh::xyzz_dbl(p);
            if ((k >> b) & 1) p = zkh::xyzz_add(p, g);
        }
        zkh::Xyzz q = p;
        for (uint32_t j = 0; j < n; j++) q = zkh::xyzz_dbl(q);
        put_affine(q, out);
    }
    return 0;
}

static int fq2_mode(const std::vector<zkh::F4>& v, FILE* out) {
    for (size_t i = 0; i < v.size(); i += 2) {
        const zkh::F2 a = {zkh::cto_mont(v[i]), zkh::cto_mont(v[i + 1])};
        const zkh::F2 sq = zkh::cfrom_mont(zkh::csqr(a)), mu = zkh::cfrom_mont(zkh::cmul(a, a));
        for (const zkh::F4* x : {&sq.c0, &sq.c1, &mu.c0, &mu.c1}) std::fwrite(x->v, 8, 4, out);
    }
    return 0;
}

int main(int argc, char** argv) {
    if (argc != 4) return 2;
    const bool curve = std::strcmp(argv[1], "g1") == 0;
    const bool fq2 = std::strcmp(argv[1], "fq2") == 0;
    const zkh::Field& F = std::strcmp(argv[1], "fr") == 0 ? zkh::fr() : zkh::fq();
    FILE* in = std::fopen(argv[2], "rb");
    if (!in) return 3;
    std::vector<zkh::F4> v;
    zkh::F4 e;
    while (std::fread(e.v, 8, 4, in) == 4) v.push_back(e);
    std::fclose(in);
    if (v.size() % 2) return 4;
    FILE* out = std::fopen(argv[3], "wb");
    if (!out) return 5;
    if (curve || fq2) {
        const int rc = curve ? curve_mode(v, out) : fq2_mode(v, out);
        std::fclose(out);
        return rc;
    }
    for (size_t i = 0; i < v.size(); i += 2) {
        const zkh::F4& a = v[i];
        const zkh::F4& b = v[i + 1];
        const zkh::F4 z = {{0, 0, 0, 0}};
        const zkh::F4 r[5] = {zkh::mul(F, a, b), zkh::is_zero(a) ? z : zkh::inv(F, a), zkh::add(F, a, b),
                              zkh::sub(F, a, b), zkh::to_mont(F, a)};
        for (const zkh::F4& x : r) std::fwrite(x.v, 8, 4, out);
    }
    std::fclose(out);
    return 0;
}

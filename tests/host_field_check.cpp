// Host build of pyzkp_gb300/csrc/host_field.hpp (the library's host-side field code: final
// MSM combination, twiddle and scale tables). Reads records of two 32-byte little-endian
// canonical elements (a, b) from argv[2] for the field named by argv[1] ("fr" or "fq") and
// writes, per record, mul(a, b), inv(a) (zero for a == 0), add(a, b), sub(a, b) and
// to_mont(a) to argv[3]. Built and checked by tests/test_host_field.py.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../pyzkp_gb300/csrc/host_field.hpp"

int main(int argc, char** argv) {
    if (argc != 4) return 2;
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

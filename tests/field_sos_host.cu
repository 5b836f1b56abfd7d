// Host build of the separated Fq forms of field.cuh (512-bit product, then one Montgomery
// reduction): the same template code the device runs, with the carry flag emulated on the
// host. Reads records of four 32-byte little-endian elements (a, b, c, d) from argv[1] and
// writes, per record, sqr(a), a b + c d, a b - c d, a b and the Fq2 product
// (a + b u)(c + d u) (two coordinates; Montgomery products, lazy values) to argv[2]. Built and
// checked by tests/test_field_sos_host.py.
#include <cstdio>
#include <vector>

#include "../pyzkp_gb300/csrc/field.cuh"

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 3;
    std::vector<zk::fe> v;
    zk::fe e;
    while (std::fread(e.v, 4, 8, in) == 8) v.push_back(e);
    std::fclose(in);
    if (v.size() % 4) return 4;
    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 5;
    for (size_t i = 0; i < v.size(); i += 4) {
        const zk::fe_pair q = zk::fe2_mul_lazy<zk::FqP>(v[i], v[i + 1], v[i + 2], v[i + 3]);
        const zk::fe r[6] = {zk::fe_sqr_sos<zk::FqP>(v[i]), zk::fe_mul_add_sos<zk::FqP>(v[i], v[i + 1], v[i + 2], v[i + 3]),
                             zk::fe_mul_sub_sos<zk::FqP>(v[i], v[i + 1], v[i + 2], v[i + 3]),
                             zk::fe_mul_sos<zk::FqP>(v[i], v[i + 1]), q.c0, q.c1};
        for (const zk::fe& x : r) std::fwrite(x.v, 4, 8, out);
    }
    std::fclose(out);
    return 0;
}

// The reference's MSM and Pedersen golden-vector checks (src/tests.cpp:6036-6142),
// restated over the C++ point API of include/helioselene_gb300.hpp: decode the
// points with from_bytes, run multi_scalar_mul / pedersen_commit on the GPU,
// compare to_bytes with the expected encoding.
//
//   golden_msm <cases file>
//
// The cases file (written by tests/test_gpu_cpp_boundary.py from
// tests/golden/vectors.json) holds whitespace-separated records:
//   msm <curve> <n> <label>  <n scalars> <n points> <result>
//   pedersen <curve> <n> <label>  <blinding> <H> <n values> <n generators> <result>
// with every 32-byte value in hex.  Prints one line per case; the exit status
// is the number of failures.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "helioselene_gb300.hpp"

namespace hg = helioselene_gb300;

static hg::ScalarBytes from_hex(const std::string &h)
{
    hg::ScalarBytes b{};
    if (h.size() != 64)
        throw std::runtime_error("bad hex value: " + h);
    for (size_t i = 0; i < 32; i++)
        b[i] = (uint8_t)std::stoul(h.substr(2 * i, 2), nullptr, 16);
    return b;
}

static std::string to_hex(const hg::ScalarBytes &b)
{
    static const char *d = "0123456789abcdef";
    std::string s;
    for (uint8_t v : b) {
        s += d[v >> 4];
        s += d[v & 15];
    }
    return s;
}

template <class P>
static std::vector<P> decode_all(std::istream &in, size_t n)
{
    std::vector<P> v;
    for (size_t i = 0; i < n; i++) {
        std::string h;
        in >> h;
        const auto b = from_hex(h);
        v.push_back(P::from_bytes(b.data()).value());  // the vectors' points are valid encodings
    }
    return v;
}

static std::vector<hg::ScalarBytes> read_scalars(std::istream &in, size_t n)
{
    std::vector<hg::ScalarBytes> v(n);
    for (size_t i = 0; i < n; i++) {
        std::string h;
        in >> h;
        v[i] = from_hex(h);
    }
    return v;
}

template <class P>
static bool run_case(std::istream &in, const std::string &kind, size_t n, std::string &got, std::string &want)
{
    if (kind == "msm") {
        const auto s = read_scalars(in, n);
        const auto p = decode_all<P>(in, n);
        got = to_hex(P::multi_scalar_mul(s.data(), p.data(), n).to_bytes());
    } else {
        std::string h;
        in >> h;
        const auto blinding = from_hex(h);
        const auto H = decode_all<P>(in, 1);
        const auto v = read_scalars(in, n);
        const auto g = decode_all<P>(in, n);
        got = to_hex(P::pedersen_commit(blinding, H[0], v.data(), g.data(), n).to_bytes());
    }
    in >> want;
    return got == want;
}

int main(int argc, char **argv)
{
    if (argc != 2) {
        std::cerr << "usage: golden_msm <cases file>\n";
        return 2;
    }
    std::ifstream in(argv[1]);
    int failures = 0, cases = 0;
    std::string kind, curve, label;
    size_t n = 0;
    try {
        while (in >> kind >> curve >> n >> label) {
            std::string got, want;
            const bool ok = curve == "helios" ? run_case<hg::HeliosPoint>(in, kind, n, got, want)
                                              : run_case<hg::SelenePoint>(in, kind, n, got, want);
            cases++;
            if (!ok)
                failures++;
            std::cout << (ok ? "ok " : "FAIL ") << curve << " " << kind << " " << label
                      << (ok ? std::string() : " got " + got + " want " + want) << "\n";
        }
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1000;
    }
    std::cout << cases << " cases, " << failures << " failures\n";
    return cases ? failures : 1000;
}

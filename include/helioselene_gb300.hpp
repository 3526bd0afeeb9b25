/*
 * helioselene_gb300.hpp -- C++17 host layer over the C ABI in helioselene_gb300.h.
 *
 * Three things, all inline over the C entry points (link -lhelioselene_gb300):
 *
 *  1. helioselene_gb300::Context -- an owning handle of hs_context with
 *     status codes turned into helioselene_gb300::Error exceptions.
 *  2. helioselene_gb300::HeliosPoint / SelenePoint -- the MSM part of the
 *     reference's C++ point API (include/helioselene_point.h:113-174 and
 *     :299-307, implemented at src/api_point.cpp:98-144): from_bytes,
 *     to_bytes, raw(), multi_scalar_mul, pedersen_commit, batch_to_affine, with
 *     the reference's semantics (n == 0 gives the identity, any 32-byte scalar
 *     is accepted).  Scalars are the 32-byte little-endian encodings that
 *     HeliosScalar::to_bytes returns.
 *  3. When the reference's own headers are included before this one, the
 *     bindings that a maintainer wires into them (the static branch of
 *     helios/include/helios_msm_vartime.h:50-60, or the dispatch-table slots of
 *     include/helioselene_dispatch.h:49-57): functions with the exact
 *     signatures of helios_msm_vartime, helios_pedersen_commit,
 *     helios_batch_to_affine, helios_scalarmult_vartime and their Selene twins,
 *     over the reference's helios_jacobian / selene_jacobian records, with
 *     compile-time checks that those records have the layout of
 *     hs_jacobian51; and, with include/helioselene_point.h, multi_scalar_mul /
 *     pedersen_commit over helioselene::HeliosPoint and HeliosScalar.
 */
#ifndef HELIOSELENE_GB300_HPP
#define HELIOSELENE_GB300_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "helioselene_gb300.h"

namespace helioselene_gb300 {

using ScalarBytes = std::array<uint8_t, 32>;

class Error : public std::runtime_error {
  public:
    Error(int status, const std::string &what) : std::runtime_error(what), status_(status) {}
    int status() const { return status_; }

  private:
    int status_;
};

inline void check(int status, const char *what, const hs_context *ctx)
{
    if (status != HS_OK) {
        const char *detail = hs_last_error(ctx);
        throw Error(status, std::string(what) + ": " + hs_strerror(status) +
                                (detail && *detail ? std::string(" (") + detail + ")" : std::string()));
    }
}

// One stream and workspace on one device; calls on one context are serialised.
class Context {
  public:
    explicit Context(int device = 0)
    {
        check(hs_context_create(&h_, device), "hs_context_create", nullptr);
    }
    ~Context()
    {
        if (h_)
            hs_context_destroy(h_);
    }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    Context(Context &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    Context &operator=(Context &&o) noexcept
    {
        if (this != &o) {
            if (h_)
                hs_context_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    hs_context *get() const { return h_; }

    // sum scalars[i] * points[i] over host records (HS_FMT_JACOBIAN51 in and out)
    hs_jacobian51 msm(int curve, const uint8_t *scalars, const hs_jacobian51 *points, size_t n) const
    {
        hs_jacobian51 r{};
        check(hs_msm(h_, curve, scalars, points, HS_FMT_JACOBIAN51, n, &r, HS_FMT_JACOBIAN51), "hs_msm", h_);
        return r;
    }
    hs_jacobian51 pedersen(int curve, const uint8_t blinding[32], const hs_jacobian51 &H, const uint8_t *values,
                           const hs_jacobian51 *generators, size_t n) const
    {
        hs_jacobian51 r{};
        check(hs_pedersen(h_, curve, blinding, &H, values, generators, HS_FMT_JACOBIAN51, n, &r, HS_FMT_JACOBIAN51),
              "hs_pedersen", h_);
        return r;
    }
    void batch_to_affine(int curve, const hs_jacobian51 *points, size_t n, hs_affine51 *out) const
    {
        if (n)
            check(hs_batch_to_affine(h_, curve, points, n, out, HS_FMT_AFFINE51), "hs_batch_to_affine", h_);
    }
    ScalarBytes compress(int curve, const hs_jacobian51 &p) const
    {
        ScalarBytes b{};
        check(hs_compress(h_, curve, &p, HS_FMT_JACOBIAN51, 1, b.data()), "hs_compress", h_);
        return b;
    }
    // nullopt for an encoding the reference rejects (src/api_point.cpp:58-64)
    std::optional<hs_jacobian51> decompress(int curve, const uint8_t bytes[32]) const
    {
        hs_jacobian51 r{};
        uint8_t valid = 0;
        const int s = hs_decompress(h_, curve, bytes, 1, &r, HS_FMT_JACOBIAN51, &valid);
        if (s == HS_EINVAL && !valid)
            return std::nullopt;
        check(s, "hs_decompress", h_);
        return r;
    }

  private:
    hs_context *h_ = nullptr;
};

// The process-wide context on device 0 that the point API below uses, created
// on first use (thread-safe).
inline Context &default_context()
{
    static Context ctx(0);
    return ctx;
}

// The reference's identity record (1:1:0) (helios/include/helios_ops.h:45-50).
inline hs_jacobian51 identity_record()
{
    hs_jacobian51 r{};
    r.X[0] = 1;
    r.Y[0] = 1;
    return r;
}

template <int CURVE>
class Point {
  public:
    Point() : jac_(identity_record()) {}
    static Point identity() { return Point(); }
    static Point from_jacobian(const hs_jacobian51 &j)
    {
        Point p;
        p.jac_ = j;
        return p;
    }
    const hs_jacobian51 &raw() const { return jac_; }
    hs_jacobian51 &raw() { return jac_; }

    static std::optional<Point> from_bytes(const uint8_t bytes[32])
    {
        const auto j = default_context().decompress(CURVE, bytes);
        if (!j)
            return std::nullopt;
        return from_jacobian(*j);
    }
    ScalarBytes to_bytes() const { return default_context().compress(CURVE, jac_); }
    bool is_identity() const { return to_bytes() == ScalarBytes{}; }
    bool operator==(const Point &o) const { return to_bytes() == o.to_bytes(); }
    bool operator!=(const Point &o) const { return !(*this == o); }

    // sum scalars[i] * points[i] (src/api_point.cpp:98-116); n == 0 gives the identity
    static Point multi_scalar_mul(const ScalarBytes *scalars, const Point *points, size_t n)
    {
        if (n == 0 || !scalars || !points)
            return Point();
        std::vector<hs_jacobian51> pts(n);
        for (size_t i = 0; i < n; i++)
            pts[i] = points[i].jac_;
        return from_jacobian(default_context().msm(CURVE, scalars[0].data(), pts.data(), n));
    }

    // blinding * H + sum values[i] * generators[i] (src/api_point.cpp:118-144)
    static Point pedersen_commit(const ScalarBytes &blinding, const Point &H, const ScalarBytes *values,
                                 const Point *generators, size_t n)
    {
        if (n == 0 || !values || !generators)
            return Point();
        std::vector<hs_jacobian51> gens(n);
        for (size_t i = 0; i < n; i++)
            gens[i] = generators[i].jac_;
        return from_jacobian(
            default_context().pedersen(CURVE, blinding.data(), H.jac_, values[0].data(), gens.data(), n));
    }

    // every point's affine form with one shared inversion; the identity gives (0,0)
    // (helios/include/helios_batch_affine.h:55-98)
    static std::vector<hs_affine51> batch_to_affine(const Point *points, size_t n)
    {
        std::vector<hs_jacobian51> in(n);
        for (size_t i = 0; i < n; i++)
            in[i] = points[i].jac_;
        std::vector<hs_affine51> out(n);
        default_context().batch_to_affine(CURVE, in.data(), n, out.data());
        return out;
    }

  private:
    hs_jacobian51 jac_;
};

static_assert(sizeof(ScalarBytes) == 32 && alignof(ScalarBytes) == 1, "scalar arrays are packed 32-byte rows");

using HeliosPoint = Point<HS_HELIOS>;
using SelenePoint = Point<HS_SELENE>;

// Layout checks of a reference record type against the ABI records.
template <class J>
constexpr bool jacobian_layout_matches()
{
    return sizeof(J) == sizeof(hs_jacobian51) && std::is_trivially_copyable<J>::value &&
           std::is_standard_layout<J>::value;
}

}  // namespace helioselene_gb300

/* ---- bindings over the reference's own types (its headers included first) ---- */
#if defined(HELIOSELENE_HELIOS_H)
#include <cstddef>
static_assert(helioselene_gb300::jacobian_layout_matches<helios_jacobian>(), "helios_jacobian layout");
static_assert(offsetof(helios_jacobian, X) == offsetof(hs_jacobian51, X) &&
                  offsetof(helios_jacobian, Y) == offsetof(hs_jacobian51, Y) &&
                  offsetof(helios_jacobian, Z) == offsetof(hs_jacobian51, Z),
              "helios_jacobian coordinates at the offsets of hs_jacobian51");
static_assert(sizeof(helios_affine) == sizeof(hs_affine51) && offsetof(helios_affine, y) == offsetof(hs_affine51, y),
              "helios_affine layout");
namespace helioselene_gb300 {
// helios/include/helios_msm_vartime.h:45-71
inline void helios_msm_vartime(helios_jacobian *result, const unsigned char *scalars, const helios_jacobian *points,
                               size_t n)
{
    hs_helios_msm_vartime(reinterpret_cast<hs_jacobian51 *>(result), scalars,
                          reinterpret_cast<const hs_jacobian51 *>(points), n);
}
// helios/include/helios_pedersen.h:55-86
inline void helios_pedersen_commit(helios_jacobian *result, const unsigned char *blinding, const helios_jacobian *H,
                                   const unsigned char *values, const helios_jacobian *generators, size_t n)
{
    hs_helios_pedersen_commit(reinterpret_cast<hs_jacobian51 *>(result), blinding,
                              reinterpret_cast<const hs_jacobian51 *>(H), values,
                              reinterpret_cast<const hs_jacobian51 *>(generators), n);
}
// helios/include/helios_batch_affine.h:55-98
inline void helios_batch_to_affine(helios_affine *out, const helios_jacobian *points, size_t n)
{
    hs_helios_batch_to_affine(reinterpret_cast<hs_affine51 *>(out), reinterpret_cast<const hs_jacobian51 *>(points),
                              n);
}
// helios/include/helios_scalarmult_vartime.h:39-57
inline void helios_scalarmult_vartime(helios_jacobian *result, const unsigned char scalar[32], const helios_jacobian *p)
{
    hs_helios_scalarmult_vartime(reinterpret_cast<hs_jacobian51 *>(result), scalar,
                                 reinterpret_cast<const hs_jacobian51 *>(p));
}
}  // namespace helioselene_gb300
#endif

#if defined(HELIOSELENE_SELENE_H)
#include <cstddef>
static_assert(helioselene_gb300::jacobian_layout_matches<selene_jacobian>(), "selene_jacobian layout");
static_assert(offsetof(selene_jacobian, X) == offsetof(hs_jacobian51, X) &&
                  offsetof(selene_jacobian, Y) == offsetof(hs_jacobian51, Y) &&
                  offsetof(selene_jacobian, Z) == offsetof(hs_jacobian51, Z),
              "selene_jacobian coordinates at the offsets of hs_jacobian51");
static_assert(sizeof(selene_affine) == sizeof(hs_affine51) && offsetof(selene_affine, y) == offsetof(hs_affine51, y),
              "selene_affine layout");
namespace helioselene_gb300 {
// selene/include/selene_msm_vartime.h (twin of helios_msm_vartime)
inline void selene_msm_vartime(selene_jacobian *result, const unsigned char *scalars, const selene_jacobian *points,
                               size_t n)
{
    hs_selene_msm_vartime(reinterpret_cast<hs_jacobian51 *>(result), scalars,
                          reinterpret_cast<const hs_jacobian51 *>(points), n);
}
inline void selene_pedersen_commit(selene_jacobian *result, const unsigned char *blinding, const selene_jacobian *H,
                                   const unsigned char *values, const selene_jacobian *generators, size_t n)
{
    hs_selene_pedersen_commit(reinterpret_cast<hs_jacobian51 *>(result), blinding,
                              reinterpret_cast<const hs_jacobian51 *>(H), values,
                              reinterpret_cast<const hs_jacobian51 *>(generators), n);
}
inline void selene_batch_to_affine(selene_affine *out, const selene_jacobian *points, size_t n)
{
    hs_selene_batch_to_affine(reinterpret_cast<hs_affine51 *>(out), reinterpret_cast<const hs_jacobian51 *>(points),
                              n);
}
inline void selene_scalarmult_vartime(selene_jacobian *result, const unsigned char scalar[32], const selene_jacobian *p)
{
    hs_selene_scalarmult_vartime(reinterpret_cast<hs_jacobian51 *>(result), scalar,
                                 reinterpret_cast<const hs_jacobian51 *>(p));
}
}  // namespace helioselene_gb300
#endif

#if defined(HELIOSELENE_API_POINT_H) && defined(HELIOSELENE_API_SCALAR_H)
namespace helioselene_gb300 {
// HeliosPoint::multi_scalar_mul / pedersen_commit (src/api_point.cpp:98-144) on the
// GPU, over the reference's own point and scalar classes
template <class RefPoint, class RefScalar>
inline RefPoint ref_multi_scalar_mul(int curve, const RefScalar *scalars, const RefPoint *points, size_t n)
{
    RefPoint r;
    if (n == 0 || !scalars || !points)
        return r;
    std::vector<unsigned char> sb(32 * n);
    std::vector<hs_jacobian51> pts(n);
    for (size_t i = 0; i < n; i++) {
        const auto b = scalars[i].to_bytes();
        std::memcpy(sb.data() + 32 * i, b.data(), 32);
        std::memcpy(&pts[i], &points[i].raw(), sizeof(hs_jacobian51));
    }
    const hs_jacobian51 out = default_context().msm(curve, sb.data(), pts.data(), n);
    std::memcpy(&r.raw(), &out, sizeof(hs_jacobian51));
    return r;
}
template <class RefPoint, class RefScalar>
inline RefPoint ref_pedersen_commit(int curve, const RefScalar &blinding, const RefPoint &H, const RefScalar *values,
                                    const RefPoint *generators, size_t n)
{
    RefPoint r;
    if (n == 0 || !values || !generators)
        return r;
    const auto bb = blinding.to_bytes();
    std::vector<unsigned char> vb(32 * n);
    std::vector<hs_jacobian51> gens(n);
    for (size_t i = 0; i < n; i++) {
        const auto b = values[i].to_bytes();
        std::memcpy(vb.data() + 32 * i, b.data(), 32);
        std::memcpy(&gens[i], &generators[i].raw(), sizeof(hs_jacobian51));
    }
    hs_jacobian51 h;
    std::memcpy(&h, &H.raw(), sizeof(h));
    const hs_jacobian51 out = default_context().pedersen(curve, bb.data(), h, vb.data(), gens.data(), n);
    std::memcpy(&r.raw(), &out, sizeof(hs_jacobian51));
    return r;
}
inline helioselene::HeliosPoint multi_scalar_mul(const helioselene::HeliosScalar *scalars,
                                                 const helioselene::HeliosPoint *points, size_t n)
{
    return ref_multi_scalar_mul(HS_HELIOS, scalars, points, n);
}
inline helioselene::SelenePoint multi_scalar_mul(const helioselene::SeleneScalar *scalars,
                                                 const helioselene::SelenePoint *points, size_t n)
{
    return ref_multi_scalar_mul(HS_SELENE, scalars, points, n);
}
inline helioselene::HeliosPoint pedersen_commit(const helioselene::HeliosScalar &blinding,
                                                const helioselene::HeliosPoint &H,
                                                const helioselene::HeliosScalar *values,
                                                const helioselene::HeliosPoint *generators, size_t n)
{
    return ref_pedersen_commit(HS_HELIOS, blinding, H, values, generators, n);
}
inline helioselene::SelenePoint pedersen_commit(const helioselene::SeleneScalar &blinding,
                                                const helioselene::SelenePoint &H,
                                                const helioselene::SeleneScalar *values,
                                                const helioselene::SelenePoint *generators, size_t n)
{
    return ref_pedersen_commit(HS_SELENE, blinding, H, values, generators, n);
}
}  // namespace helioselene_gb300
#endif

#endif /* HELIOSELENE_GB300_HPP */

// Drop-in counterpart of MRMD's datatypes.hpp (datatypes.hpp:91-224) on top of
// the mrmd_gb300 C ABI.  Only the types the LJ / AdResS hot path uses are
// provided: real_t, idx_t, Point3D, AXIS, the predicate forms and
// HalfVerletList.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "mrmd_gb300.h"

namespace mrmd
{
using idx_t = int64_t;
using real_t = double;
using Point3D = std::array<real_t, 3>;
using Vector3D = std::array<real_t, 3>;

constexpr real_t operator""_r(const long double val) { return static_cast<real_t>(val); }
constexpr real_t operator""_r(const unsigned long long val) { return static_cast<real_t>(val); }

enum class AXIS : idx_t
{
    X = 0,
    Y = 1,
    Z = 2
};

// Errors of the C ABI surface as exceptions (the reference aborts through
// MRMD_HOST_CHECK; an exception keeps that "stop here" behaviour catchable).
class Error : public std::runtime_error
{
public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
    int code;
};

// The drop-in's own helpers live in mrmd::gb300, a namespace the reference
// does not use (its mrmd::*::impl namespaces hold its own internals, such as
// action::impl::CoulombDSF).
namespace gb300
{
inline mrmd_ctx* context();  // process-wide context on device 0 (initialization.cpp:23-44)

inline void check(int rc, const char* what)
{
    if (rc != MRMD_OK) throw Error(rc, std::string(what) + ": " + mrmd_ctx_last_error(context()));
}

inline mrmd_ctx* context()
{
    static mrmd_ctx* ctx = []
    {
        mrmd_ctx* c = nullptr;
        if (mrmd_ctx_create(&c, 0) != MRMD_OK) throw Error(MRMD_ERR_CUDA, "cannot create the mrmd_gb300 context");
        return c;
    }();
    return ctx;
}
}  // namespace gb300

// Two-position predicates for LennardJones::apply_if: the in-tree callers use
// util::IsInSymmetricSlab combined with || or && (examples/04:206-227).
struct TwoPositionsPredicate
{
    mrmd_pred p{MRMD_PRED_ALWAYS, 0, 0.0, 0.0, 0.0, 0.0};
};

// HalfVerletList (datatypes.hpp:184-187): Cabana half list, device-resident.
class HalfVerletList
{
public:
    HalfVerletList() { gb300::check(mrmd_nlist_init(gb300::context(), &list_), "HalfVerletList"); }
    ~HalfVerletList() { mrmd_nlist_free(gb300::context(), &list_); }
    HalfVerletList(const HalfVerletList&) = delete;
    HalfVerletList& operator=(const HalfVerletList&) = delete;

    // build(positions, begin, end, cutoff, cell_ratio, gridMin, gridMax, maxNeigh)
    // (examples/02_LennardJones_NVE.cpp:156-163); `positions` is the device
    // position array of an Atoms or Molecules object with `numPositions` entries.
    void build(const double* positions, idx_t numPositions, idx_t begin, idx_t end, real_t cutoff,
               real_t cellRatio, const real_t* gridMin, const real_t* gridMax, idx_t maxNeigh = 60)
    {
        gb300::check(mrmd_nlist_build(gb300::context(), &list_, positions, numPositions, begin, end, cutoff,
                                     cellRatio, gridMin, gridMax, maxNeigh),
                    "HalfVerletList::build");
    }

    idx_t numPairs() const { return list_.totalPairs; }
    const mrmd_nlist* raw() const { return &list_; }

private:
    mrmd_nlist list_{};
};
}  // namespace mrmd

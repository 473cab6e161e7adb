// Drop-in counterpart of io/DumpThermoForce.hpp: the table text of
// io/DumpThermoForce.cpp:24-64 (bin centres, then one force line per type).
#pragma once

#include <string>

#include "../action/AdResS.hpp"

namespace mrmd
{
namespace io
{
inline void dumpThermoForce(const std::string& filename, const action::ThermodynamicForce& thermodynamicForce,
                            const idx_t& typeId)
{
    impl::check(mrmd_tf_dump(impl::context(), thermodynamicForce.raw(), filename.c_str(), typeId),
                "dumpThermoForce");
}

inline void dumpThermoForce(const std::string& filename, const action::ThermodynamicForce& thermodynamicForce)
{
    impl::check(mrmd_tf_dump(impl::context(), thermodynamicForce.raw(), filename.c_str(), -1), "dumpThermoForce");
}
}  // namespace io
}  // namespace mrmd

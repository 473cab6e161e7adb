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
    gb300::check(mrmd_tf_dump(gb300::context(), thermodynamicForce.raw(), filename.c_str(), typeId),
                "dumpThermoForce");
}

inline void dumpThermoForce(const std::string& filename, const action::ThermodynamicForce& thermodynamicForce)
{
    gb300::check(mrmd_tf_dump(gb300::context(), thermodynamicForce.raw(), filename.c_str(), -1), "dumpThermoForce");
}
}  // namespace io
}  // namespace mrmd

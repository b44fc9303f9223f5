// Stand-in for the run identifier: a fixed string (the cross-check writes no
// files that need a unique name).
#pragma once
#include <string>
namespace boost { namespace uuids {
struct uuid {};
struct random_generator { uuid operator()() const { return uuid{}; } };
inline std::string to_string(const uuid&) { return "00000000-0000-0000-0000-000000000000"; }
} }

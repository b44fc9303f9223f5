// Stand-in for boost::property_tree::ptree: the reference's XML parameter
// reader (setup.cpp) is not compiled for the cross-check, but setup.h, which
// its potential factory includes, names these members.  An empty tree.
#pragma once
#include <cstddef>
#include <stdexcept>
#include <string>
#include <boost/optional.hpp>

namespace boost { namespace property_tree {
class ptree {
  public:
    std::size_t count(const std::string&) const { return 0; }
    template <class T> T get(const std::string&) const { throw std::logic_error("empty parameter tree"); }
    boost::optional<const ptree&> get_child_optional(const std::string&) const { return {}; }
};
} }

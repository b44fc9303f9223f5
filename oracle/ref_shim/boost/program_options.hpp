// A minimal stand-in for boost::program_options::variables_map as the
// reference reads it (params["name"].as<T>(), .empty(), count), filled by
// the cross-check harness instead of a command line.  Not Boost code.
#pragma once
#include <any>
#include <map>
#include <string>

namespace boost { namespace program_options {

class variable_value {
    std::any v_;
  public:
    variable_value() = default;
    template <class T>
    explicit variable_value(const T& v) : v_(v) {}
    template <class T>
    variable_value(const T& v, bool) : v_(v) {}
    bool empty() const { return !v_.has_value(); }
    template <class T> const T& as() const { return std::any_cast<const T&>(v_); }
    template <class T> T& as() { return std::any_cast<T&>(v_); }
    const std::any& value() const { return v_; }
    std::any& value() { return v_; }
};

// Declarations that setup.h names; the command-line parser itself is not
// part of the cross-check build.
class options_description {};
template <class T, class charT = char>
class typed_value {
  public:
    typed_value* default_value(const T&) { return this; }
};
template <class T> typed_value<T>* value() { return nullptr; }

class variables_map : public std::map<std::string, variable_value> {
  public:
    using std::map<std::string, variable_value>::operator[];
    const variable_value& operator[](const std::string& k) const {
        static const variable_value none;
        auto it = find(k);
        return it == end() ? none : it->second;
    }
    template <class T> void set(const std::string& k, const T& v) { std::map<std::string, variable_value>::operator[](k) = variable_value(v); }
};

inline void notify(variables_map&) {}

} }

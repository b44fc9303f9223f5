// A minimal stand-in for boost::format, enough for the reference's headers
// and estimator files in the cross-check build: printf-style directives
// (%[flags][width][.precision]conversion, %% for a literal percent) filled
// left to right by operator%.  Not Boost code.
#pragma once
#include <cstdio>
#include <ostream>
#include <sstream>
#include <string>
#include <type_traits>

namespace boost {

class format {
  public:
    explicit format(const std::string& f) : fmt_(f) { advance(); }
    explicit format(const char* f) : fmt_(f) { advance(); }

    template <class T>
    format& operator%(const T& v) {
        if (spec_.empty()) return *this;          // more arguments than directives
        out_ += render(spec_, v);
        advance();
        return *this;
    }
    std::string str() const { return out_ + fmt_.substr(pos_); }
    friend std::ostream& operator<<(std::ostream& os, const format& f) { return os << f.str(); }

  private:
    std::string fmt_, out_, spec_;
    size_t pos_ = 0;

    // copy literal text up to the next directive and cut the directive out
    void advance() {
        spec_.clear();
        while (pos_ < fmt_.size()) {
            const size_t p = fmt_.find('%', pos_);
            if (p == std::string::npos) { out_ += fmt_.substr(pos_); pos_ = fmt_.size(); return; }
            out_ += fmt_.substr(pos_, p - pos_);
            if (p + 1 < fmt_.size() && fmt_[p + 1] == '%') { out_ += '%'; pos_ = p + 2; continue; }
            size_t q = p + 1;
            while (q < fmt_.size() && std::string("-+ #0123456789.").find(fmt_[q]) != std::string::npos) ++q;
            while (q < fmt_.size() && std::string("hlLqjzt").find(fmt_[q]) != std::string::npos) ++q;
            if (q >= fmt_.size()) { out_ += fmt_.substr(p); pos_ = fmt_.size(); return; }
            spec_ = fmt_.substr(p, q - p + 1);
            pos_ = q + 1;
            return;
        }
    }
    static std::string strip_length(std::string s) {
        std::string r;
        for (char c : s) if (std::string("hlLqjzt").find(c) == std::string::npos) r += c;
        return r;
    }
    template <class T>
    static std::string render(const std::string& spec, const T& v) {
        char buf[512];
        const char conv = spec.back();
        const std::string base = strip_length(spec.substr(0, spec.size() - 1));
        if constexpr (std::is_floating_point<T>::value) {
            if (conv == 'd' || conv == 'i' || conv == 's')
                std::snprintf(buf, sizeof buf, (base + "g").c_str(), (double)v);
            else
                std::snprintf(buf, sizeof buf, (base + conv).c_str(), (double)v);
            return buf;
        } else if constexpr (std::is_integral<T>::value) {
            if (conv == 'f' || conv == 'e' || conv == 'E' || conv == 'g' || conv == 'G')
                std::snprintf(buf, sizeof buf, (base + conv).c_str(), (double)v);
            else if (conv == 's')
                std::snprintf(buf, sizeof buf, (base + "lld").c_str(), (long long)v);
            else if (std::is_signed<T>::value)
                std::snprintf(buf, sizeof buf, (base + "ll" + conv).c_str(), (long long)v);
            else
                std::snprintf(buf, sizeof buf, (base + "ll" + conv).c_str(), (unsigned long long)v);
            return buf;
        } else {
            std::ostringstream os;
            os << v;
            std::snprintf(buf, sizeof buf, (base + "s").c_str(), os.str().c_str());
            return buf;
        }
    }
};

inline std::string str(const format& f) { return f.str(); }

}  // namespace boost

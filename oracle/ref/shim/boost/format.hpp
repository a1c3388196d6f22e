// Stand-in for boost::format, enough for the "%i" file names the kinematic-chain demo header builds.
#pragma once
#include <sstream>
#include <string>
namespace boost {
class format {
public:
    explicit format(const char *f) : f_(f) {}
    template <class T> format &operator%(const T &v) {
        std::ostringstream o; o << v;
        auto p = f_.find('%');
        if (p != std::string::npos) { auto e = p + 1; while (e < f_.size() && !isalpha((unsigned char)f_[e])) ++e; f_.replace(p, e - p + 1, o.str()); }
        return *this;
    }
    std::string str() const { return f_; }
private:
    std::string f_;
};
inline std::string str(const format &f) { return f.str(); }
}

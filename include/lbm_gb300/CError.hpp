// CError.hpp -- the string error sink of the reference (src/lib/CError.hpp):
// messages are piped in with <<, `error()` is true once anything was written,
// getString() returns the text.
#ifndef LBM_GB300_CERROR_HPP
#define LBM_GB300_CERROR_HPP

#include <sstream>
#include <string>

class CError {
    std::ostringstream os_;
    bool set_ = false;

public:
    static std::ostream &endl(std::ostream &o) { return o << std::endl; }
    bool operator()() const { return set_; }
    template <typename V>
    CError &operator<<(const V &v) {
        os_ << v;
        set_ = true;
        return *this;
    }
    CError &operator<<(std::ostream &(*pf)(std::ostream &)) {
        os_ << pf;
        set_ = true;
        return *this;
    }
    std::string getString() const { return os_.str(); }
    void clear() {
        os_.str("");
        set_ = false;
    }
};

#endif

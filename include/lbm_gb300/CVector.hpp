// CVector.hpp -- the small fixed-size vectors the reference's interfaces use
// (src/libmath/CVector3.hpp, CVector4.hpp): CVector<3,int>, CVector<3,T>,
// CVector<4,T> with the members those interfaces call.
#ifndef LBM_GB300_CVECTOR_HPP
#define LBM_GB300_CVECTOR_HPP

#include <cmath>
#include <ostream>

template <int D, typename T>
class CVector {
public:
    T data[D];

    CVector() {
        for (int i = 0; i < D; i++) data[i] = T(0);
    }
    explicit CVector(const T x) {
        for (int i = 0; i < D; i++) data[i] = x;
    }
    CVector(const T x0, const T x1, const T x2) {
        static_assert(D == 3, "three components");
        data[0] = x0; data[1] = x1; data[2] = x2;
    }
    CVector(const T x0, const T x1, const T x2, const T x3) {
        static_assert(D == 4, "four components");
        data[0] = x0; data[1] = x1; data[2] = x2; data[3] = x3;
    }
    explicit CVector(const T v[D]) {
        for (int i = 0; i < D; i++) data[i] = v[i];
    }
    template <typename U>
    explicit CVector(const CVector<D, U> &v) {
        for (int i = 0; i < D; i++) data[i] = T(v.data[i]);
    }

    T &operator[](int i) { return data[i]; }
    const T &operator[](int i) const { return data[i]; }

    /** number of cells of a box with these edge lengths */
    T elements() const {
        T e = T(1);
        for (int i = 0; i < D; i++) e *= data[i];
        return e;
    }
    T dotProd(const CVector &v) const {
        T s = T(0);
        for (int i = 0; i < D; i++) s += data[i] * v.data[i];
        return s;
    }
    T length() const {
        T s = T(0);
        for (int i = 0; i < D; i++) s += data[i] * data[i];
        return std::sqrt(s);
    }
    T max() const {
        T m = data[0];
        for (int i = 1; i < D; i++) m = data[i] > m ? data[i] : m;
        return m;
    }

    CVector operator+(const CVector &v) const { CVector r; for (int i = 0; i < D; i++) r.data[i] = data[i] + v.data[i]; return r; }
    CVector operator-(const CVector &v) const { CVector r; for (int i = 0; i < D; i++) r.data[i] = data[i] - v.data[i]; return r; }
    CVector operator*(const T a) const { CVector r; for (int i = 0; i < D; i++) r.data[i] = data[i] * a; return r; }
    CVector operator/(const T a) const { CVector r; for (int i = 0; i < D; i++) r.data[i] = data[i] / a; return r; }
    CVector &operator+=(const CVector &v) { for (int i = 0; i < D; i++) data[i] += v.data[i]; return *this; }
    CVector &operator-=(const CVector &v) { for (int i = 0; i < D; i++) data[i] -= v.data[i]; return *this; }
    CVector &operator*=(const T a) { for (int i = 0; i < D; i++) data[i] *= a; return *this; }
    CVector &operator/=(const T a) { for (int i = 0; i < D; i++) data[i] /= a; return *this; }
    bool operator==(const CVector &v) const { for (int i = 0; i < D; i++) if (data[i] != v.data[i]) return false; return true; }
    bool operator!=(const CVector &v) const { return !(*this == v); }
};

template <int D, typename T>
std::ostream &operator<<(std::ostream &o, const CVector<D, T> &v) {
    o << "[";
    for (int i = 0; i < D; i++) o << (i ? ", " : "") << v.data[i];
    return o << "]";
}

#endif

// CDomain.hpp -- one subdomain: id, size in cells, origin in the global
// grid, physical length (src/CDomain.hpp:17-57, same constructors and getters).
#ifndef LBM_GB300_CDOMAIN_HPP
#define LBM_GB300_CDOMAIN_HPP

#include "CVector.hpp"

template <typename T>
class CDomain {
    int _UID;
    CVector<3, int> _size;
    CVector<3, int> _origin_cell;
    CVector<3, T> _length;

public:
    CDomain(int UID, CVector<3, int> size, CVector<3, int> origin_cell, CVector<3, T> length)
        : _UID(UID), _size(size), _origin_cell(origin_cell), _length(length) {}
    CDomain(int UID, CVector<3, int> size)
        : _UID(UID), _size(size), _origin_cell(0, 0, 0), _length(T(0.05), T(0.05), T(0.05)) {}

    CVector<3, int> getOrigin() const { return _origin_cell; }
    CVector<3, int> getSize() const { return _size; }
    int getUid() const { return _UID; }
    CVector<3, T> getLength() const { return _length; }
};

#endif

// CComm.hpp -- descriptor of one face exchange (src/CComm.hpp:20-77): the
// destination subdomain, send/receive sizes and origins and the inward
// direction.  In this build the destination is a subdomain index of the
// same process, not an MPI rank.
#ifndef LBM_GB300_CCOMM_HPP
#define LBM_GB300_CCOMM_HPP

#include "CVector.hpp"

template <typename T>
class CComm {
    int _dstID;
    CVector<3, int> _send_size, _recv_size, _send_origin, _recv_origin, _comm_direction;

public:
    CComm(int dstID, CVector<3, int> send_size, CVector<3, int> recv_size, CVector<3, int> send_origin,
          CVector<3, int> recv_origin, CVector<3, int> comm_direction)
        : _dstID(dstID), _send_size(send_size), _recv_size(recv_size), _send_origin(send_origin),
          _recv_origin(recv_origin), _comm_direction(comm_direction) {}

    CVector<3, int> getCommDirection() const { return _comm_direction; }
    void setCommDirection(CVector<3, int> normal) { _comm_direction = normal; }
    CVector<3, int> getRecvOrigin() const { return _recv_origin; }
    void setRecvOrigin(CVector<3, int> o) { _recv_origin = o; }
    CVector<3, int> getRecvSize() const { return _recv_size; }
    void setRecvSize(CVector<3, int> s) { _recv_size = s; }
    CVector<3, int> getSendOrigin() const { return _send_origin; }
    void setSendOrigin(CVector<3, int> o) { _send_origin = o; }
    CVector<3, int> getSendSize() const { return _send_size; }
    void setSendSize(CVector<3, int> s) { _send_size = s; }
    int getDstId() const { return _dstID; }
    void setDstId(int d) { _dstID = d; }
    /** axis of the exchange (0 x, 1 y, 2 z) */
    int axis() const { return _comm_direction[0] != 0 ? 0 : _comm_direction[1] != 0 ? 1 : 2; }
};

#endif

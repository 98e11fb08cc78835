// frames.hpp - the properties.msgpack.bin frames of beRTAMC2D
// (data::msgpack_pack and saver::save_frame, src/beyondRTA_MC2d.cpp:1604-1769):
// each frame is "<byte count>#" followed by a msgpack array
//   [time, Eeff, [temperature per box], then per box either
//    (2*nnz, [mode, count, mode, count, ...]) or (0, [42.0])]
// with integers in their smallest msgpack encoding; the file ends with "0#".
#pragma once

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace bte {

class MsgPack {
public:
    std::string buf;
    void array(std::size_t n) {
        if (n < 16) {
            put(uint8_t(0x90 | n));
        } else if (n <= 0xffff) {
            put(0xdc);
            be(uint64_t(n), 2);
        } else {
            put(0xdd);
            be(uint64_t(n), 4);
        }
    }
    void f64(double x) {
        uint64_t b;
        std::memcpy(&b, &x, 8);
        put(0xcb);
        be(b, 8);
    }
    void uint(uint64_t v) {
        if (v < 128) {
            put(uint8_t(v));
        } else if (v <= 0xff) {
            put(0xcc);
            be(v, 1);
        } else if (v <= 0xffff) {
            put(0xcd);
            be(v, 2);
        } else if (v <= 0xffffffffull) {
            put(0xce);
            be(v, 4);
        } else {
            put(0xcf);
            be(v, 8);
        }
    }
    void sint(int64_t v) {
        if (v >= 0) {
            uint(uint64_t(v));
        } else if (v >= -32) {
            put(uint8_t(0xe0 | (v + 32)));
        } else if (v >= -128) {
            put(0xd0);
            be(uint64_t(v), 1);
        } else if (v >= -32768) {
            put(0xd1);
            be(uint64_t(v), 2);
        } else if (v >= -2147483648ll) {
            put(0xd2);
            be(uint64_t(v), 4);
        } else {
            put(0xd3);
            be(uint64_t(v), 8);
        }
    }

private:
    void put(uint8_t c) { buf.push_back(char(c)); }
    void be(uint64_t v, int bytes) {
        for (int i = bytes - 1; i >= 0; --i) put(uint8_t(v >> (8 * i)));
    }
};

// One frame: histogram H is [nboxes][nmodes].
inline std::string berta_frame(double time, double Eeff, const std::vector<double>& temperatures,
                               const int* H, std::size_t nboxes, std::size_t nmodes) {
    MsgPack pk;
    pk.array(3 + 2 * nboxes);
    pk.f64(time);
    pk.f64(Eeff);
    pk.array(temperatures.size());
    for (double t : temperatures) pk.f64(t);
    for (std::size_t b = 0; b < nboxes; ++b) {
        std::size_t nz = 0;
        for (std::size_t k = 0; k < nmodes; ++k) nz += H[b * nmodes + k] != 0;
        if (nz == 0) {
            pk.uint(0);
            pk.array(1);
            pk.f64(42.0);
            continue;
        }
        pk.uint(2 * nz);
        pk.array(2 * nz);
        for (std::size_t k = 0; k < nmodes; ++k) {
            const int v = H[b * nmodes + k];
            if (v != 0) {
                pk.uint(k);
                pk.sint(v);
            }
        }
    }
    return std::to_string(pk.buf.size()) + "#" + pk.buf;
}

}  // namespace bte

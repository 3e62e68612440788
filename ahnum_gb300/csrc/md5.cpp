// MD5 as specified in RFC 1321, section 3: 64-byte blocks, four rounds of sixteen steps,
// T[i] = floor(2^32 |sin(i + 1)|), little-endian words and length.
#include "md5.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace kg {

namespace {

struct Tables {
    uint32_t T[64];
    Tables() {
        for (int i = 0; i < 64; i++) T[i] = (uint32_t)std::floor(std::fabs(std::sin((double)(i + 1))) * 4294967296.0);
    }
};

const Tables &tables() {
    static const Tables t;
    return t;
}

inline uint32_t rotl(uint32_t x, int s) { return (x << s) | (x >> (32 - s)); }

// per-round shift amounts (RFC 1321 3.4)
constexpr int kShift[4][4] = {{7, 12, 17, 22}, {5, 9, 14, 20}, {4, 11, 16, 23}, {6, 10, 15, 21}};

}  // namespace

Md5::Md5() : h_{0x67452301u, 0xefcdab89u, 0x98badcfeu, 0x10325476u} {}

void Md5::block(const uint8_t *p) {
    uint32_t X[16];
    for (int i = 0; i < 16; i++)
        X[i] = (uint32_t)p[4 * i] | (uint32_t)p[4 * i + 1] << 8 | (uint32_t)p[4 * i + 2] << 16 |
               (uint32_t)p[4 * i + 3] << 24;
    const uint32_t *T = tables().T;
    uint32_t a = h_[0], b = h_[1], c = h_[2], d = h_[3];
    for (int i = 0; i < 64; i++) {
        const int round = i / 16;
        uint32_t f;
        int idx;
        switch (round) {
        case 0: f = (b & c) | (~b & d); idx = i; break;
        case 1: f = (b & d) | (c & ~d); idx = (5 * i + 1) & 15; break;
        case 2: f = b ^ c ^ d; idx = (3 * i + 5) & 15; break;
        default: f = c ^ (b | ~d); idx = (7 * i) & 15; break;
        }
        const uint32_t next = b + rotl(a + f + X[idx] + T[i], kShift[round][i & 3]);
        a = d;
        d = c;
        c = b;
        b = next;
    }
    h_[0] += a;
    h_[1] += b;
    h_[2] += c;
    h_[3] += d;
}

void Md5::update(const void *data, size_t len) {
    const uint8_t *p = static_cast<const uint8_t *>(data);
    bytes_ += len;
    while (len) {
        const size_t take = std::min(len, sizeof buf_ - fill_);
        std::memcpy(buf_ + fill_, p, take);
        fill_ += take;
        p += take;
        len -= take;
        if (fill_ == sizeof buf_) {
            block(buf_);
            fill_ = 0;
        }
    }
}

void Md5::digest(uint8_t out[16]) {
    const uint64_t bits = bytes_ * 8;
    const uint8_t one = 0x80, zero = 0;
    update(&one, 1);
    while (fill_ != 56) update(&zero, 1);
    uint8_t len[8];
    for (int i = 0; i < 8; i++) len[i] = (uint8_t)(bits >> (8 * i));
    update(len, 8);
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = (uint8_t)(h_[i] >> (8 * j));
}

std::string Md5::hex(const void *data, size_t len) {
    Md5 m;
    m.update(data, len);
    uint8_t d[16];
    m.digest(d);
    static const char *digits = "0123456789abcdef";
    std::string s(32, '0');
    for (int i = 0; i < 16; i++) {
        s[2 * i] = digits[d[i] >> 4];
        s[2 * i + 1] = digits[d[i] & 15];
    }
    return s;
}

}  // namespace kg

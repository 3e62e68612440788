// MD5 (RFC 1321), for the PRST proof files' hashes, fingerprints and .md5 sidecars.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

namespace kg {

class Md5 {
  public:
    Md5();
    void update(const void *data, size_t len);
    void digest(uint8_t out[16]);  // finishes; the object must not be updated afterwards
    static std::string hex(const void *data, size_t len);  // lowercase, 32 characters

  private:
    void block(const uint8_t *p);
    uint32_t h_[4];
    uint64_t bytes_ = 0;
    uint8_t buf_[64];
    size_t fill_ = 0;
};

}  // namespace kg

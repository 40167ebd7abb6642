// Keccak-256 (the Keccak SHA-3 submission with its original padding, as used by Ethereum):
// the sponge over Keccak-f[1600] with rate 136 bytes, capacity 512 bits and the pad10*1 rule
// with domain byte 0x01.  sha3_256 is the same sponge with the FIPS 202 domain byte 0x06; it
// exists so the permutation can be checked against any SHA3-256 implementation.
#pragma once
#include <stddef.h>
#include <stdint.h>

namespace gkrgpu {

void keccak256(const uint8_t* in, size_t len, uint8_t out[32]);
void sha3_256(const uint8_t* in, size_t len, uint8_t out[32]);

}  // namespace gkrgpu

/* Test infrastructure only: the transcript hash of the oracle.
 *
 * SHA-256 (gkr_oracle.c, the reference's transcript hash) by default; Keccak-256 after
 * oracle_set_fs_hash(1), the Keccak256 member of the reference's FiatShamir_hash_type
 * (include/configuration/config.hpp:18-24), which the reference names but does not
 * implement.  Keccak-f[1600] is written here from its definition, independently of the
 * product's copy; SHA3-256 (the same sponge with the FIPS 202 domain byte) is exported so
 * the tests can check the permutation against Python's hashlib.
 */
#include <stdint.h>
#include <string.h>

#include "gkr_oracle.h"

static int g_fs_hash = 0;

void oracle_set_fs_hash(int h) { g_fs_hash = h; }
int oracle_get_fs_hash(void) { return g_fs_hash; }

static uint64_t rol64(uint64_t v, int n) { return n ? (v << n) | (v >> (64 - n)) : v; }

static void keccak_f1600(uint64_t s[5][5]) {
    static uint64_t rc[24];
    static int rho[5][5];
    static int ready = 0;
    if (!ready) {
        /* round constants: bit 2^j - 1 of RC[i] is the LFSR output rc(j + 7 i) */
        uint8_t lfsr = 1;
        int bits[168];
        for (int t = 0; t < 168; t++) {
            bits[t] = lfsr & 1;
            lfsr = (uint8_t)((lfsr << 1) ^ ((lfsr & 0x80) ? 0x71 : 0));
        }
        for (int i = 0; i < 24; i++) {
            rc[i] = 0;
            for (int j = 0; j < 7; j++) rc[i] |= (uint64_t)bits[j + 7 * i] << ((1 << j) - 1);
        }
        /* rotation offsets along the pi walk from (1, 0) */
        int x = 1, y = 0;
        rho[0][0] = 0;
        for (int t = 0; t < 24; t++) {
            rho[x][y] = ((t + 1) * (t + 2) / 2) % 64;
            int nx = y, ny = (2 * x + 3 * y) % 5;
            x = nx;
            y = ny;
        }
        ready = 1;
    }
    for (int r = 0; r < 24; r++) {
        uint64_t c[5], d[5], b[5][5];
        for (int x = 0; x < 5; x++) c[x] = s[x][0] ^ s[x][1] ^ s[x][2] ^ s[x][3] ^ s[x][4];
        for (int x = 0; x < 5; x++) d[x] = c[(x + 4) % 5] ^ rol64(c[(x + 1) % 5], 1);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) s[x][y] ^= d[x];
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) b[y][(2 * x + 3 * y) % 5] = rol64(s[x][y], rho[x][y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) s[x][y] = b[x][y] ^ (~b[(x + 1) % 5][y] & b[(x + 2) % 5][y]);
        s[0][0] ^= rc[r];
    }
}

static void sponge(const uint8_t* in, uint64_t len, uint8_t pad, uint8_t out[32]) {
    uint64_t s[5][5];
    uint8_t block[136];
    memset(s, 0, sizeof(s));
    for (;;) {
        uint64_t take = len < 136 ? len : 136;
        memset(block, 0, sizeof(block));
        memcpy(block, in, take);
        int last = take < 136;
        if (last) {
            block[take] ^= pad;
            block[135] ^= 0x80;
        }
        for (int i = 0; i < 17; i++) {
            uint64_t w = 0;
            for (int k = 0; k < 8; k++) w |= (uint64_t)block[8 * i + k] << (8 * k);
            s[i % 5][i / 5] ^= w;
        }
        keccak_f1600(s);
        if (last) break;
        in += 136;
        len -= 136;
    }
    for (int i = 0; i < 4; i++)
        for (int k = 0; k < 8; k++) out[8 * i + k] = (uint8_t)(s[i % 5][i / 5] >> (8 * k));
}

void oracle_keccak256(const uint8_t* in, uint64_t len, uint8_t out[32]) { sponge(in, len, 0x01, out); }
void oracle_sha3_256(const uint8_t* in, uint64_t len, uint8_t out[32]) { sponge(in, len, 0x06, out); }

void oracle_fs_hash(const uint8_t* in, uint64_t len, uint8_t out[32]) {
    if (g_fs_hash == 1)
        oracle_keccak256(in, len, out);
    else
        oracle_sha256(in, len, out);
}

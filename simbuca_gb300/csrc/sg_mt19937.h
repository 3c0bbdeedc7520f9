// sg_mt19937.h -- the 32-bit Mersenne Twister MT19937 (Matsumoto & Nishimura, ACM
// TOMACS 8(1), 1998) with its published 32-bit seeding; uniform() returns the 32-bit
// output times 2^-32 in [0, 1), the conversion of the reference's MTRand
// (bin/mtrand.h:102-104).  Host only: the reference's draws are sequential.
#pragma once
#include <cstdint>

class SgMt19937 {
public:
    explicit SgMt19937(uint32_t s) {
        st_[0] = s;
        for (int i = 1; i < N; i++) st_[i] = 1812433253u * (st_[i - 1] ^ (st_[i - 1] >> 30)) + (uint32_t)i;
        pos_ = N;
    }
    uint32_t next() {
        if (pos_ == N) twist();
        uint32_t y = st_[pos_++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        return y ^ (y >> 18);
    }
    double uniform() { return (double)next() * (1.0 / 4294967296.0); }

private:
    static constexpr int N = 624, M = 397;
    static uint32_t mix(uint32_t u, uint32_t v) {
        const uint32_t y = (u & 0x80000000u) | (v & 0x7fffffffu);
        return (y >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
    }
    void twist() {
        for (int i = 0; i < N; i++) st_[i] = st_[(i + M) % N] ^ mix(st_[i], st_[(i + 1) % N]);
        pos_ = 0;
    }
    uint32_t st_[N];
    int pos_;
};

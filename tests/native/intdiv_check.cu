// Host check of the integer-pipe division in hsr_device.cuh: the same
// ip_recip / ip_quot / ip_div_ok code, compiled for the host, against the
// host's IEEE double division on seeded operand sets (random significands
// and exponents, divisor significands near 1 and near 2, dividends equal or
// next to the divisor).  Prints "<sets on the integer path> <mismatches>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "../../hsrq3in_gb300/csrc/hsr_device.cuh"

using namespace hsr;

static unsigned long long bits_of(double x) {
    unsigned long long u;
    std::memcpy(&u, &x, 8);
    return u;
}
static double double_of(unsigned long long u) {
    double x;
    std::memcpy(&x, &u, 8);
    return x;
}

int main(int argc, char **argv) {
    const long long N = argc > 1 ? std::atoll(argv[1]) : 20000000LL;
    std::mt19937_64 rng(20261204ULL);
    long long fast = 0, bad = 0;
    for (long long i = 0; i < N; ++i) {
        const unsigned long long ra = rng(), rb = rng(), rc = rng();
        const int mode = (int)(i % 8);
        unsigned long long fa = ra & kSigMask, fb = rb & kSigMask;
        if (mode == 1) fb |= 0xffffffffff000ULL;
        if (mode == 2) fb &= 0xffULL;
        if (mode == 3) fa = fb;
        if (mode == 4) fa = (fb + ((rc >> 8) & 0xf)) & kSigMask;
        if (mode == 5) fa = (fb - ((rc >> 8) & 0xf)) & kSigMask;
        if (mode == 6) fa |= 0xfffffffffff00ULL;
        int ea = 1023 + (int)((rc >> 16) % 200) - 100, eb = 1023 + (int)((rc >> 32) % 200) - 100;
        if (mode == 7) {
            ea = 1 + (int)((rc >> 16) % 2046);
            eb = 1 + (int)((rc >> 32) % 2046);
        }
        const unsigned long long sign = ((rc >> 60) & 1ULL) << 63;
        const double a = double_of(sign | ((unsigned long long)ea << 52) | fa);
        const double b = double_of(((unsigned long long)eb << 52) | fb);
        if (!ip_div_ok(ea, eb, fb)) continue;   // these take the FP64 instruction
        ++fast;
        const unsigned long long mb = fb | kHidden;
        const double q = double_of(ip_quot(fa | kHidden, mb, ip_recip(mb), ea - eb + 1023, sign));
        if (bits_of(q) != bits_of(a / b)) {
            if (bad < 5) std::printf("mismatch a=%a b=%a got=%a want=%a\n", a, b, q, a / b);
            ++bad;
        }
    }
    std::printf("%lld %lld\n", fast, bad);
    return bad != 0;
}

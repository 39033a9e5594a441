// zstd_host.cpp — the page decoder of slothdb_gb300/csrc/gb_zstd.h built for
// the host, so that the CPU tests can check it against another ZSTD
// implementation on the same frames (tests/test_zstd_cpu.py).
#include <cstdlib>

#include "gb_zstd.h"

extern "C" long long zstd_host_decompress(const unsigned char *src, long long n, unsigned char *dst, long long cap) {
    gbz::ZsScratch *S = (gbz::ZsScratch *)malloc(sizeof(gbz::ZsScratch));
    if (!S) return -2;
    const long long r = gbz::zstd_decompress(src, n, dst, cap, *S);
    free(S);
    return r;
}

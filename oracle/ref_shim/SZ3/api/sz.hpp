/* Declaration-only stand-in for SZ3's API header (see mpi.h two directories up). */
#pragma once
#include <stddef.h>
namespace SZ3 {
enum EB { EB_ABS, EB_REL };
enum ALGO { ALGO_LORENZO_REG, ALGO_INTERP_LORENZO, ALGO_INTERP };
struct Config {
    Config(int, int, int);
    EB errorBoundMode;
    ALGO cmprAlgo;
    double absErrorBound;
};
}
template <class T> char *SZ_compress(const SZ3::Config &, const T *, size_t &);
template <class T> void SZ_decompress(const SZ3::Config &, const char *, size_t, T *);

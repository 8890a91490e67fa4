// encode.cpp -- host encoder / decoder of the reference's edit files.
//
// _deltas.bin: the per-voxel delta symbols (0..q) packed LSB-first with
//   bits_for_max(q) bits each (pack_nbits / bits_for_max, pMSz.cu:2328-2356),
//   then zstd level 5 (compress_symbols_0_N, pMSz.cu:2359-2369, called with
//   level 5 at pMSz.cu:2480).
// _edits.bin: the clamp values as raw T bytes, zstd level 3 (compress_zstd,
//   pMSz.cu:2261-2277, called at pMSz.cu:2473); empty input gives an empty
//   file, as compress_zstd returns {} for an empty vector.
// Both go through the system libzstd.so.1 (the image ships no zstd.h, so the
// handful of public zstd entry points used are declared below).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pmsz_host.h"

extern "C" {
size_t ZSTD_compress(void *dst, size_t dstCapacity, const void *src, size_t srcSize, int compressionLevel);
size_t ZSTD_compressBound(size_t srcSize);
unsigned ZSTD_isError(size_t code);
const char *ZSTD_getErrorName(size_t code);
size_t ZSTD_decompress(void *dst, size_t dstCapacity, const void *src, size_t compressedSize);
unsigned long long ZSTD_getFrameContentSize(const void *src, size_t srcSize);
unsigned ZSTD_versionNumber(void);
}

namespace pmsz {
int set_error(int status, const std::string &msg);
}

namespace {

unsigned bits_for_max(unsigned m) {  // pMSz.cu:2352-2356
    if (m == 0) return 1;
    return static_cast<unsigned>(std::ceil(std::log2(static_cast<double>(m) + 1.0)));
}

int zstd_to_malloc(const void *src, size_t n, int level, uint8_t **out, size_t *out_len) {
    const size_t cap = ZSTD_compressBound(n);
    uint8_t *buf = static_cast<uint8_t *>(std::malloc(cap ? cap : 1));
    if (!buf) return pmsz::set_error(PMSZ_ERR_OOM, "encoder buffer allocation failed");
    const size_t c = ZSTD_compress(buf, cap, src, n, level);
    if (ZSTD_isError(c)) {
        std::free(buf);
        return pmsz::set_error(PMSZ_ERR_ARG, std::string("zstd compression failed: ") + ZSTD_getErrorName(c));
    }
    *out = buf;
    *out_len = c;
    return PMSZ_OK;
}

}  // namespace

extern "C" int pmsz_encode_deltas(const uint8_t *deltas, size_t n, int q, uint8_t **out, size_t *out_len) {
    if (!deltas || !out || !out_len || q < 1 || q > 255) return pmsz::set_error(PMSZ_ERR_ARG, "bad encoder arguments");
    const unsigned nbits = bits_for_max(static_cast<unsigned>(q));
    if (nbits > 8) return pmsz::set_error(PMSZ_ERR_ARG, "symbol width above 8 bits");
    std::vector<uint8_t> packed;
    packed.reserve((n * nbits + 7) / 8);
    const uint64_t mask = (1ull << nbits) - 1ull;
    uint64_t buf = 0;
    unsigned cnt = 0;
    for (size_t i = 0; i < n; ++i) {  // pack_nbits, pMSz.cu:2328-2348
        const uint64_t v = deltas[i];
        if (v > mask) return pmsz::set_error(PMSZ_ERR_ARG, "delta symbol exceeds 0..q");
        buf |= (v & mask) << cnt;
        cnt += nbits;
        while (cnt >= 8) {
            packed.push_back(static_cast<uint8_t>(buf & 0xFF));
            buf >>= 8;
            cnt -= 8;
        }
    }
    if (cnt) packed.push_back(static_cast<uint8_t>(buf & 0xFF));
    return zstd_to_malloc(packed.data(), packed.size(), 5, out, out_len);
}

extern "C" int pmsz_encode_packed_deltas(const uint8_t *packed, size_t len, uint8_t **out, size_t *out_len) {
    if ((!packed && len) || !out || !out_len) return pmsz::set_error(PMSZ_ERR_ARG, "bad encoder arguments");
    return zstd_to_malloc(packed, len, 5, out, out_len);
}

extern "C" int pmsz_encode_clamps(const void *values, size_t count, size_t elem_size, uint8_t **out,
                                  size_t *out_len) {
    if (!out || !out_len || (count && !values) || (elem_size != 4 && elem_size != 8))
        return pmsz::set_error(PMSZ_ERR_ARG, "bad encoder arguments");
    if (count == 0) {
        *out = nullptr;
        *out_len = 0;
        return PMSZ_OK;
    }
    return zstd_to_malloc(values, count * elem_size, 3, out, out_len);
}

extern "C" int pmsz_decode_deltas(const uint8_t *comp, size_t len, size_t n, int q, uint8_t *deltas) {
    if ((!comp && len) || (!deltas && n) || q < 1 || q > 255) return pmsz::set_error(PMSZ_ERR_ARG, "bad decoder arguments");
    const unsigned nbits = bits_for_max(static_cast<unsigned>(q));
    const size_t need = (n * nbits + 7) / 8;
    std::vector<uint8_t> packed(need ? need : 1);
    const size_t got = ZSTD_decompress(packed.data(), need, comp, len);
    if (ZSTD_isError(got) || got != need) return pmsz::set_error(PMSZ_ERR_ARG, "deltas stream has the wrong size or is corrupt");
    const uint64_t mask = (1ull << nbits) - 1ull;
    uint64_t buf = 0;
    unsigned cnt = 0;
    size_t pos = 0;
    for (size_t i = 0; i < n; ++i) {  // unpack_nbits, pMSz.cu:2393-2410
        while (cnt < nbits) {
            buf |= static_cast<uint64_t>(packed[pos++]) << cnt;
            cnt += 8;
        }
        deltas[i] = static_cast<uint8_t>(buf & mask);
        buf >>= nbits;
        cnt -= nbits;
    }
    return PMSZ_OK;
}

extern "C" int pmsz_decode_clamps(const uint8_t *comp, size_t len, size_t elem_size, void **values, size_t *count) {
    if (!values || !count || (elem_size != 4 && elem_size != 8)) return pmsz::set_error(PMSZ_ERR_ARG, "bad decoder arguments");
    if (len == 0) {
        *values = nullptr;
        *count = 0;
        return PMSZ_OK;
    }
    const unsigned long long sz = ZSTD_getFrameContentSize(comp, len);
    if (sz >= 0xFFFFFFFFFFFFFFFEull || sz % elem_size) return pmsz::set_error(PMSZ_ERR_ARG, "clamp stream has no valid size");
    void *buf = std::malloc(sz ? sz : 1);
    if (!buf) return pmsz::set_error(PMSZ_ERR_OOM, "decoder allocation failed");
    const size_t got = ZSTD_decompress(buf, sz, comp, len);
    if (ZSTD_isError(got) || got != sz) {
        std::free(buf);
        return pmsz::set_error(PMSZ_ERR_ARG, "clamp stream is corrupt");
    }
    *values = buf;
    *count = sz / elem_size;
    return PMSZ_OK;
}

extern "C" void pmsz_free(void *p) { std::free(p); }

extern "C" unsigned pmsz_zstd_version(void) { return ZSTD_versionNumber(); }

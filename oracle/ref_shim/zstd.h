/* Prototypes of the five public libzstd 1.5 functions the reference coder
 * calls (HuffmanZSTDCoder.cuh:359-392); the library itself is the system's
 * libzstd.so.1.  Test infrastructure for oracle/ref_harness.cu only. */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
size_t ZSTD_compressBound(size_t srcSize);
size_t ZSTD_compress(void *dst, size_t dstCapacity, const void *src, size_t srcSize, int compressionLevel);
size_t ZSTD_decompress(void *dst, size_t dstCapacity, const void *src, size_t compressedSize);
unsigned ZSTD_isError(size_t code);
const char *ZSTD_getErrorName(size_t code);
#ifdef __cplusplus
}
#endif

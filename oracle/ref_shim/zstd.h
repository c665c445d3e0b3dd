/*
 * Declaration-only stand-in for the public zstd API, used ONLY by
 * oracle/build_ref.sh to compile the reference CPU sources (which include
 * "zstd.h") against the system runtime library libzstd.so.1, which ships
 * without headers in this image.  It declares exactly the symbols those
 * sources call; the values of the two parameter enumerators are zstd's
 * documented stable ABI values.
 *
 * The reference includes this header from inside a C++ namespace, so it
 * must not include any system header itself and must give the functions C
 * linkage.
 */
#ifndef GFAZ_ORACLE_ZSTD_SHIM_H
#define GFAZ_ORACLE_ZSTD_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ZSTD_CCtx_s ZSTD_CCtx;

typedef enum {
  ZSTD_c_compressionLevel = 100,
  ZSTD_c_nbWorkers = 400
} ZSTD_cParameter;

ZSTD_CCtx *ZSTD_createCCtx(void);
size_t ZSTD_freeCCtx(ZSTD_CCtx *cctx);
size_t ZSTD_CCtx_setParameter(ZSTD_CCtx *cctx, ZSTD_cParameter param,
                              int value);
size_t ZSTD_compressBound(size_t srcSize);
size_t ZSTD_compress2(ZSTD_CCtx *cctx, void *dst, size_t dstCapacity,
                      const void *src, size_t srcSize);
size_t ZSTD_decompress(void *dst, size_t dstCapacity, const void *src,
                       size_t compressedSize);
unsigned ZSTD_isError(size_t code);
const char *ZSTD_getErrorName(size_t code);
unsigned ZSTD_versionNumber(void);

#ifdef __cplusplus
}
#endif

#endif

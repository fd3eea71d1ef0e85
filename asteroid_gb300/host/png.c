/*
 * png.c -- the PNG writer of the ANIMATE frames (host, C); the role of write_PNGs'
 * per-snapshot file (misc.c:372-460), which the reference writes with libpng.
 *
 * An 8-bit RGB image (colour type 2, no interlace, filter 0 on every row): signature, IHDR,
 * one IDAT holding a zlib stream of the rows, IEND, each chunk with its CRC-32 (ISO 3309
 * polynomial, as the PNG specification gives it).  Built with zlib (AST_HAVE_ZLIB) the stream is
 * deflated at zlib's default level, as libpng does by default; without it the stream is made of
 * stored deflate blocks (RFC 1951 section 3.2.4) closed by the Adler-32 of the rows (RFC 1950).
 * Either file decodes to the same pixels.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "asteroid_gb300.h"
#include "host_internal.h"
#ifdef AST_HAVE_ZLIB
#include <zlib.h>
#endif

static uint32_t crc_table[256];
static int crc_ready = 0;

static void crc_init(void)
{
    for (uint32_t n = 0; n < 256; n++) {
        uint32_t c = n;
        for (int k = 0; k < 8; k++) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = 1;
}

static uint32_t crc_update(uint32_t crc, const unsigned char* p, size_t n)
{
    for (size_t i = 0; i < n; i++) crc = crc_table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
    return crc;
}

static void put32(unsigned char* p, uint32_t v)
{
    p[0] = (unsigned char)(v >> 24); p[1] = (unsigned char)(v >> 16);
    p[2] = (unsigned char)(v >> 8); p[3] = (unsigned char)v;
}

static int write_chunk(FILE* fp, const char* type, const unsigned char* data, size_t n)
{
    unsigned char h[8];
    put32(h, (uint32_t)n);
    memcpy(h + 4, type, 4);
    uint32_t crc = crc_update(0xffffffffu, (const unsigned char*)type, 4);
    crc = crc_update(crc, data, n) ^ 0xffffffffu;
    unsigned char t[4];
    put32(t, crc);
    return fwrite(h, 1, 8, fp) == 8 && (n == 0 || fwrite(data, 1, n, fp) == n) && fwrite(t, 1, 4, fp) == 4;
}

#ifndef AST_HAVE_ZLIB
/* zlib stream of stored blocks (at most 65535 bytes each). */
static unsigned char* stored_stream(const unsigned char* src, size_t n, size_t* out_n)
{
    const size_t blocks = n / 65535 + 1;
    unsigned char* out = (unsigned char*)malloc(2 + n + 5 * blocks + 4);
    if (!out) return NULL;
    size_t k = 0;
    out[k++] = 0x78; /* CM 8, CINFO 7 */
    out[k++] = 0x01; /* no dictionary, fastest; (0x78 << 8 | 0x01) % 31 == 0 */
    size_t i = 0;
    do {
        const size_t len = n - i > 65535 ? 65535 : n - i;
        out[k++] = (i + len == n) ? 1 : 0; /* BFINAL, BTYPE 00 */
        out[k++] = (unsigned char)len; out[k++] = (unsigned char)(len >> 8);
        out[k++] = (unsigned char)~len; out[k++] = (unsigned char)(~len >> 8);
        memcpy(out + k, src + i, len);
        k += len;
        i += len;
    } while (i < n);
    uint32_t a = 1, b = 0;
    for (size_t j = 0; j < n; j++) {
        a = (a + src[j]) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(out + k, (b << 16) | a);
    *out_n = k + 4;
    return out;
}
#endif

int ast_write_png(const char* path, const uint8_t* rgb, int32_t width, int32_t height)
{
    if (!path || !rgb || width <= 0 || height <= 0 || width > 65536 || height > 65536)
        return ast_set_error(AST_E_INVALID, "ast_write_png: bad argument");
    if (!crc_ready) crc_init();
    const size_t row = 1 + 3 * (size_t)width, n = row * (size_t)height;
    unsigned char* raw = (unsigned char*)malloc(n);
    if (!raw) return ast_set_error(AST_E_NOMEM, "ast_write_png: out of host memory");
    for (int32_t y = 0; y < height; y++) {
        raw[row * y] = 0; /* filter type None */
        memcpy(raw + row * y + 1, rgb + 3 * (size_t)width * y, 3 * (size_t)width);
    }
    unsigned char* z = NULL;
    size_t zn = 0;
#ifdef AST_HAVE_ZLIB
    uLongf cap = compressBound((uLong)n);
    z = (unsigned char*)malloc(cap);
    if (z && compress2(z, &cap, raw, (uLong)n, Z_DEFAULT_COMPRESSION) == Z_OK) zn = cap;
    else { free(z); z = NULL; }
#else
    z = stored_stream(raw, n, &zn);
#endif
    free(raw);
    if (!z) return ast_set_error(AST_E_NOMEM, "ast_write_png: compression failed");
    FILE* fp = fopen(path, "wb");
    if (!fp) {
        free(z);
        return ast_set_error(AST_E_IO, "Could not open file %s for writing", path);
    }
    static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
    unsigned char ihdr[13];
    put32(ihdr, (uint32_t)width);
    put32(ihdr + 4, (uint32_t)height);
    ihdr[8] = 8;  /* bit depth */
    ihdr[9] = 2;  /* colour type RGB */
    ihdr[10] = 0; /* deflate */
    ihdr[11] = 0; /* adaptive filtering, filter type per row */
    ihdr[12] = 0; /* no interlace */
    int ok = fwrite(sig, 1, 8, fp) == 8 && write_chunk(fp, "IHDR", ihdr, 13) && write_chunk(fp, "IDAT", z, zn) &&
             write_chunk(fp, "IEND", NULL, 0);
    ok = (fclose(fp) == 0) && ok;
    free(z);
    return ok ? AST_OK : ast_set_error(AST_E_IO, "ast_write_png: writing %s failed", path);
}

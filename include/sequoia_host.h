/* sequoia_host.h -- host-side entry points of the drop-in: the OBJ loader and
 * the BMP writer that sit either side of the build/trace path.
 *
 * Both are plain C over plain pointers, exported from the same shared library
 * as sequoia_gpu.h (libsequoia_gpu.so).  Neither touches a GPU.
 */
#ifndef SEQUOIA_HOST_H
#define SEQUOIA_HOST_H

#include <stdint.h>

#include "sequoia_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Summary of one OBJ parse. */
typedef struct sq_obj_info {
    uint32_t faces;      /* triangles produced (a quad gives two)             */
    uint32_t vertices;   /* "v" records read                                   */
    uint32_t lines;      /* input lines as the reference reads them: one per
                            fgets() call of at most 255 characters            */
    uint32_t threads;    /* threads the parse used                            */
} sq_obj_info;

/* Replaces loadOBJFromFile (src/main.cpp:108-179) and its tokeniser gstrtok
 * (src/main.cpp:88-106).  Produces exactly the triangles the reference produces
 * for every input the reference accepts:
 *   - a line is what fgets() with a 256-byte buffer returns, so a longer line
 *     is read as several lines;
 *   - the first token of a line ends at ' ', '\t', '\n' or '\r'; later tokens
 *     at ' ', '\t' or '\n'; two delimiters in a row give an empty token; a
 *     token that reaches the end of the line without a delimiter is absent;
 *   - "v x y z": each value is (float)atof(token);
 *   - "f a b c [d]": each index is atoi(token) (so "7/2/9" reads 7), made
 *     zero-based (i - 1), or relative to the vertices read so far when
 *     negative; a fourth index adds the triangle (a, c, d); further indices
 *     are ignored;
 *   - every other line is ignored.
 * Where the reference's behaviour is undefined -- a "v" or "f" line that is
 * missing a token (it passes NULL to atof/atoi) or a face index outside the
 * vertex list (it reads out of bounds) -- this returns SQ_ERR_INVALID with
 * the line number in sq_host_last_error().  A file that cannot be opened or
 * read gives SQ_ERR_INVALID as well (the reference prints and exits).
 *
 * threads: 0 = all hardware threads.  The file is split at line boundaries
 * and parsed in parallel; the result does not depend on the thread count.
 * *tris is allocated with malloc (release it with sq_obj_free); it is NULL
 * when the file has no faces.  info may be NULL.                             */
sq_status sq_obj_load(const char* path, uint32_t threads, sq_triangle** tris, uint32_t* tri_count,
                      sq_obj_info* info);
/* The same parse over a buffer in memory (len bytes; need not be
 * NUL-terminated).                                                           */
sq_status sq_obj_parse(const char* text, uint64_t len, uint32_t threads, sq_triangle** tris,
                       uint32_t* tri_count, sq_obj_info* info);
void sq_obj_free(sq_triangle* tris);

/* Replaces the reference's image output (src/main.cpp:335-336:
 * stbi_flip_vertically_on_write(true) then stbi_write_bmp(path, w, h, 3,
 * rgb)): an uncompressed 24-bit BMP whose first image row (top of the
 * picture) is rgb row 0, rows padded to 4 bytes.  rgb: w*h*3 bytes, row
 * major, R G B.                                                             */
sq_status sq_bmp_write(const char* path, uint32_t w, uint32_t h, const uint8_t* rgb);
/* The same file image into a caller buffer of sq_bmp_size(w, h) bytes.      */
uint64_t sq_bmp_size(uint32_t w, uint32_t h);
sq_status sq_bmp_encode(uint32_t w, uint32_t h, const uint8_t* rgb, uint8_t* out);

/* Message of the last failing sq_obj_* / sq_bmp_* call on this thread.     */
const char* sq_host_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* SEQUOIA_HOST_H */

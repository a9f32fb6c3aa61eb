/*
 * voidray_assets.h — host-side asset decoding of the GB300 backend: images
 * and OBJ meshes.  Neither part needs a CUDA device.  Shares vr_status and
 * vr_last_error() with voidray_gpu.h.
 *
 * Images.  voidray reads textures and environment maps with the `image`
 * crate (`image::open(path).unwrap().to_rgb32f()`,
 * voidray_renderer/src/core/texture.rs:36-37; image 0.24.3, JPEG through
 * jpeg-decoder) and its demo scenes ship their albedo maps as JPEG
 * (voidray_app/src/examples/mushroom.rs:9-17).  A Rust caller keeps its own
 * decoder and passes float RGB to vr_scene_create; these entry points serve
 * hosts without one (the Python layer's ImageTexture.from_file).
 * Decoded: Huffman-coded DCT JPEG (ITU-T T.81 baseline, extended sequential
 * and progressive), 8-bit samples, 1 (grey), 3 (YCbCr or RGB) or 4 (Adobe
 * CMYK / YCCK) components, any sampling factors, restart intervals.  Not
 * decoded (VR_ERR_UNSUPPORTED): lossless, hierarchical and arithmetic-coded
 * frames, 12-bit samples, DNL-defined heights, images above 2^28 pixels.
 * Corrupt or truncated data returns VR_ERR_INVALID.
 *
 * Meshes.  Mesh::from_file (voidray_renderer/src/core/mesh.rs:46-74) loads
 * with obj-rs 0.7.0 as `load_obj::<TexturedVertex, u32>`; vr_obj_parse
 * restates that crate's published behaviour for this vertex type:
 *  - `v x y z [w]`, `vt u [v [w]]` (a missing v is 0), `vn x y z`; numbers
 *    are decimal (or inf / nan) read to the nearest double, then rounded to
 *    float;
 *  - `f` lines of exactly three corners `p/t/n`, all three indices present,
 *    1-based, negative ones counting back from the current end of their
 *    list; anything else fails the load, as the crate's UntriangulatedModel /
 *    InsufficientData errors do;
 *  - each distinct (position, normal, texture) triple becomes one vertex,
 *    numbered in order of first use;
 *  - other statements (o, g, s, usemtl, mtllib, l, p) and text after `#` are
 *    ignored; lines end at \n, \r\n or \r; tokens are separated by ASCII
 *    whitespace.
 * Errors name the line: "OBJ line N: ...".
 */
#ifndef VOIDRAY_ASSETS_H
#define VOIDRAY_ASSETS_H

#include <stddef.h>
#include <stdint.h>

#include "voidray_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum vr_image_format {
    VR_IMAGE_UNKNOWN = 0,
    VR_IMAGE_JPEG = 1
} vr_image_format;

typedef struct vr_image_info {
    uint32_t width;
    uint32_t height;
    uint32_t components;   /* colour components in the stream (1, 3 or 4)   */
    uint32_t format;       /* vr_image_format                                 */
    uint32_t progressive;  /* 1 for a progressive JPEG                        */
    uint32_t reserved;
} vr_image_info;

/* Reads the headers up to the frame header: size and layout, no pixels. */
vr_status vr_image_info_get(const uint8_t* data, size_t size, vr_image_info* info);

/* Decodes the whole stream to interleaved RGB8, rows top to bottom
 * (width * height * 3 bytes; `capacity` is the size of `rgb` in bytes). */
vr_status vr_image_decode_rgb8(const uint8_t* data, size_t size, uint8_t* rgb, size_t capacity);

/* Undoes the PNG scanline filters (None, Sub, Up, Average, Paeth; ISO/IEC
 * 15948 clause 9) of `rows` scanlines of `stride` bytes, each preceded by its
 * filter-type byte, read from `data` (`size` bytes, at least rows * (stride +
 * 1)).  `bpp` is the filters' byte distance: the bytes of one complete pixel,
 * at least 1.  Writes rows * stride bytes to `out`.  An unknown filter type
 * returns VR_ERR_INVALID. */
vr_status vr_png_unfilter(const uint8_t* data, size_t size, uint32_t rows, uint32_t stride, uint32_t bpp,
                          uint8_t* out);

/* TIFF 6.0 LZW (compression 5): MSB-first codes of 9-12 bits, Clear = 256,
 * end of information = 257, the code width growing one code early (at 511,
 * 1023 and 2047 table entries).  Decodes the whole of `src` (to its end of
 * information or its last whole code), writes the first `capacity` bytes of
 * the result to `out` and the result's full length to `*length`.  A code
 * that names no table entry returns VR_ERR_INVALID. */
vr_status vr_tiff_lzw_decode(const uint8_t* src, size_t size, uint8_t* out, size_t capacity, size_t* length);

/* A parsed OBJ mesh; the arrays belong to the library until vr_obj_free. */
typedef struct vr_obj_mesh {
    float* positions;      /* 3 * num_vertices                                 */
    float* uvs;            /* 2 * num_vertices                                 */
    float* normals;        /* 3 * num_vertices                                 */
    uint32_t* indices;     /* 3 * num_triangles                                */
    uint32_t num_vertices;
    uint32_t num_triangles;
} vr_obj_mesh;

/* Parses OBJ text (`size` bytes, need not be NUL-terminated) into `mesh`.
 * On failure `mesh` holds no arrays. */
vr_status vr_obj_parse(const char* text, size_t size, vr_obj_mesh* mesh);

/* Frees the arrays of a mesh vr_obj_parse filled and zeroes it. */
vr_status vr_obj_free(vr_obj_mesh* mesh);

#ifdef __cplusplus
}
#endif

#endif /* VOIDRAY_ASSETS_H */

/*
 * voidray_image.h — host-side image decoding of the GB300 backend.
 *
 * voidray reads textures and environment maps with the `image` crate
 * (`image::open(path).unwrap().to_rgb32f()`,
 * voidray_renderer/src/core/texture.rs:36-37; image 0.24.3, JPEG through
 * jpeg-decoder) and its demo scenes ship their albedo maps as JPEG
 * (voidray_app/src/examples/mushroom.rs:9-17).  A Rust caller keeps its own
 * decoder and passes float RGB to vr_scene_create; these entry points serve
 * hosts without one (the Python layer's ImageTexture.from_file).
 *
 * Decoded: Huffman-coded DCT JPEG (ITU-T T.81 baseline, extended sequential
 * and progressive), 8-bit samples, 1 (grey), 3 (YCbCr or RGB) or 4 (Adobe
 * CMYK / YCCK) components, any sampling factors, restart intervals.  Not
 * decoded (VR_ERR_UNSUPPORTED): lossless, hierarchical and arithmetic-coded
 * frames, 12-bit samples, DNL-defined heights, images above 2^28 pixels.
 * Corrupt or truncated data returns VR_ERR_INVALID.  Neither call needs a
 * CUDA device.  Shares vr_status and vr_last_error() with voidray_gpu.h.
 */
#ifndef VOIDRAY_IMAGE_H
#define VOIDRAY_IMAGE_H

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

#ifdef __cplusplus
}
#endif

#endif /* VOIDRAY_IMAGE_H */

// Declaration-only stand-in for libjpeg. The reference's image readers and
// writers (texture_mapper.h, camera.cc) reference these names; they are never
// called on the traced path (io_stubs.cc defines them so the library loads).
#pragma once
#include <cstdio>
typedef unsigned char JSAMPLE;
typedef JSAMPLE *JSAMPROW;
typedef JSAMPROW *JSAMPARRAY;
#ifndef TRUE
#define TRUE 1
#endif
struct jpeg_error_mgr { int unused; };
struct jpeg_decompress_struct {
    jpeg_error_mgr *err;
    unsigned int output_width, output_height, image_width, image_height, output_scanline;
    int num_components;
};
jpeg_error_mgr *jpeg_std_error(jpeg_error_mgr *);
void jpeg_create_decompress(jpeg_decompress_struct *);
void jpeg_stdio_src(jpeg_decompress_struct *, FILE *);
int jpeg_read_header(jpeg_decompress_struct *, int);
int jpeg_start_decompress(jpeg_decompress_struct *);
unsigned int jpeg_read_scanlines(jpeg_decompress_struct *, JSAMPARRAY, unsigned int);
int jpeg_finish_decompress(jpeg_decompress_struct *);
void jpeg_destroy_decompress(jpeg_decompress_struct *);
enum J_COLOR_SPACE { JCS_UNKNOWN, JCS_GRAYSCALE, JCS_RGB };
struct jpeg_compress_struct {
    jpeg_error_mgr *err;
    unsigned int image_width, image_height, next_scanline;
    int input_components;
    J_COLOR_SPACE in_color_space;
};
void jpeg_create_compress(jpeg_compress_struct *);
void jpeg_stdio_dest(jpeg_compress_struct *, FILE *);
void jpeg_set_defaults(jpeg_compress_struct *);
void jpeg_set_quality(jpeg_compress_struct *, int, int);
void jpeg_start_compress(jpeg_compress_struct *, int);
unsigned int jpeg_write_scanlines(jpeg_compress_struct *, JSAMPARRAY, unsigned int);
void jpeg_finish_compress(jpeg_compress_struct *);
void jpeg_destroy_compress(jpeg_compress_struct *);

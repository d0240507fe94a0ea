// Declaration-only stand-in for libjpeg. The reference's inline image readers
// reference these names; they are never called on the traced path, so no
// definitions are provided or needed.
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

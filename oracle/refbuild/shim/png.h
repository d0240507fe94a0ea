// Declaration-only stand-in for libpng. The reference's image readers and
// writers (texture_mapper.h, camera.cc) reference these names; they are never
// called on the traced path (io_stubs.cc defines them so the library loads).
#pragma once
#include <cstdio>
#include <csetjmp>
typedef struct png_struct_def png_struct; typedef png_struct *png_structp; typedef png_struct **png_structpp;
typedef struct png_info_def png_info; typedef png_info *png_infop; typedef png_info **png_infopp;
typedef unsigned char png_byte; typedef png_byte *png_bytep; typedef png_bytep *png_bytepp;
typedef unsigned int png_uint_32; typedef std::size_t png_size_t;
#define PNG_LIBPNG_VER_STRING "shim"
#define PNG_COLOR_TYPE_RGB 2
#define PNG_COLOR_TYPE_RGBA 6
#define PNG_COLOR_TYPE_RGB_ALPHA 6
#define PNG_COLOR_TYPE_GRAY 0
#define PNG_COLOR_TYPE_PALETTE 3
#define PNG_COLOR_TYPE_GRAY_ALPHA 4
#define PNG_INTERLACE_NONE 0
#define PNG_COMPRESSION_TYPE_BASE 0
#define PNG_FILTER_TYPE_BASE 0
jmp_buf &png_jmpbuf(png_structp);
int png_sig_cmp(png_bytep, png_size_t, png_size_t);
png_structp png_create_read_struct(const char *, void *, void *, void *);
png_structp png_create_write_struct(const char *, void *, void *, void *);
png_infop png_create_info_struct(png_structp);
void png_init_io(png_structp, FILE *);
void png_set_sig_bytes(png_structp, int);
void png_read_info(png_structp, png_infop);
png_uint_32 png_get_image_width(png_structp, png_infop);
png_uint_32 png_get_image_height(png_structp, png_infop);
png_byte png_get_color_type(png_structp, png_infop);
png_byte png_get_bit_depth(png_structp, png_infop);
int png_set_interlace_handling(png_structp);
void png_read_update_info(png_structp, png_infop);
png_size_t png_get_rowbytes(png_structp, png_infop);
void png_read_image(png_structp, png_bytepp);
void png_destroy_read_struct(png_structpp, png_infopp, png_infopp);
#define PNG_COMPRESSION_TYPE_DEFAULT 0
#define PNG_FILTER_TYPE_DEFAULT 0
void png_destroy_write_struct(png_structpp, png_infopp);
void png_set_IHDR(png_structp, png_infop, png_uint_32, png_uint_32, int, int, int, int, int);
void png_write_info(png_structp, png_infop);
void png_write_image(png_structp, png_bytepp);
void png_write_end(png_structp, png_infop);

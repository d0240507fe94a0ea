// Definitions of the image-I/O and FFT names that the reference's camera.cc,
// picture_functions.cc and texture readers reference (declared in shim/).  TEST INFRASTRUCTURE
// ONLY: the harness never writes or reads image files nor enables the glare
// filter, so none of these is ever called; each aborts if it were.
#include <cstdlib>
#include <cstdio>
#include <csetjmp>
#include "fftw3.h"
extern "C" {
#include <jpeglib.h>
#include <png.h>
#include <tga.h>
TGA *TGAOpen(char *, const char *) { std::abort(); }
int TGAReadImage(TGA *, TGAData *) { std::abort(); }
int TGAWriteImage(TGA *, TGAData *) { std::abort(); }
void TGAClose(TGA *) { std::abort(); }
jmp_buf &png_jmpbuf(png_structp) { std::abort(); }
int png_sig_cmp(png_bytep, png_size_t, png_size_t) { std::abort(); }
png_structp png_create_read_struct(const char *, void *, void *, void *) { std::abort(); }
png_structp png_create_write_struct(const char *, void *, void *, void *) { std::abort(); }
png_infop png_create_info_struct(png_structp) { std::abort(); }
void png_init_io(png_structp, FILE *) { std::abort(); }
void png_set_sig_bytes(png_structp, int) { std::abort(); }
void png_read_info(png_structp, png_infop) { std::abort(); }
png_uint_32 png_get_image_width(png_structp, png_infop) { std::abort(); }
png_uint_32 png_get_image_height(png_structp, png_infop) { std::abort(); }
png_byte png_get_color_type(png_structp, png_infop) { std::abort(); }
png_byte png_get_bit_depth(png_structp, png_infop) { std::abort(); }
int png_set_interlace_handling(png_structp) { std::abort(); }
void png_read_update_info(png_structp, png_infop) { std::abort(); }
png_size_t png_get_rowbytes(png_structp, png_infop) { std::abort(); }
void png_read_image(png_structp, png_bytepp) { std::abort(); }
void png_destroy_read_struct(png_structpp, png_infopp, png_infopp) { std::abort(); }
void png_destroy_write_struct(png_structpp, png_infopp) { std::abort(); }
void png_set_IHDR(png_structp, png_infop, png_uint_32, png_uint_32, int, int, int, int, int) { std::abort(); }
void png_write_info(png_structp, png_infop) { std::abort(); }
void png_write_image(png_structp, png_bytepp) { std::abort(); }
void png_write_end(png_structp, png_infop) { std::abort(); }
jpeg_error_mgr *jpeg_std_error(jpeg_error_mgr *) { std::abort(); }
void jpeg_create_decompress(jpeg_decompress_struct *) { std::abort(); }
void jpeg_stdio_src(jpeg_decompress_struct *, FILE *) { std::abort(); }
int jpeg_read_header(jpeg_decompress_struct *, int) { std::abort(); }
int jpeg_start_decompress(jpeg_decompress_struct *) { std::abort(); }
unsigned int jpeg_read_scanlines(jpeg_decompress_struct *, JSAMPARRAY, unsigned int) { std::abort(); }
int jpeg_finish_decompress(jpeg_decompress_struct *) { std::abort(); }
void jpeg_destroy_decompress(jpeg_decompress_struct *) { std::abort(); }
void jpeg_create_compress(jpeg_compress_struct *) { std::abort(); }
void jpeg_stdio_dest(jpeg_compress_struct *, FILE *) { std::abort(); }
void jpeg_set_defaults(jpeg_compress_struct *) { std::abort(); }
void jpeg_set_quality(jpeg_compress_struct *, int, int) { std::abort(); }
void jpeg_start_compress(jpeg_compress_struct *, int) { std::abort(); }
unsigned int jpeg_write_scanlines(jpeg_compress_struct *, JSAMPARRAY, unsigned int) { std::abort(); }
void jpeg_finish_compress(jpeg_compress_struct *) { std::abort(); }
void jpeg_destroy_compress(jpeg_compress_struct *) { std::abort(); }
void *fftwf_malloc(size_t n) { std::abort(); }
void fftwf_free(void *p) { std::abort(); }
void fftwf_execute(const fftwf_plan p) { std::abort(); }
void fftwf_destroy_plan(fftwf_plan p) { std::abort(); }
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags) { std::abort(); }
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *out, unsigned flags) { std::abort(); }
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany, float *in, const int *inembed, int istride, int idist, fftwf_complex *out, const int *onembed, int ostride, int odist, unsigned flags) { std::abort(); }
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany, fftwf_complex *in, const int *inembed, int istride, int idist, float *out, const int *onembed, int ostride, int odist, unsigned flags) { std::abort(); }
}

// The case-insensitive comparison of the Boost.StringAlgo stand-in
// (shim/boost/algorithm/string.hpp), used by the reference's picture loader.
#include <cctype>
#include <string>
#include "boost/algorithm/string.hpp"
namespace boost {
bool iequals(const std::string &a, const std::string &b)
{
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i)
        if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
    return true;
}
}  // namespace boost

// boost::filesystem::extension of the Boost.Filesystem stand-in
// (shim/boost/filesystem.hpp): the last '.' and what follows it.
#include "boost/filesystem.hpp"
namespace boost {
namespace filesystem {
std::string extension(const std::string &p)
{
    const size_t dot = p.find_last_of('.');
    const size_t slash = p.find_last_of('/');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return std::string();
    return p.substr(dot);
}
}  // namespace filesystem
}  // namespace boost

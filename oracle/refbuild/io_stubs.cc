// Definitions of the image-I/O and FFT names that the reference's camera.cc,
// picture_functions.cc and texture readers reference (declared in shim/).  TEST INFRASTRUCTURE
// ONLY: the harness never writes or reads image files, so the image-I/O
// functions abort if called; the FFT functions compute (below).
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
// FFTW's single-precision interface (fftw3.h as FFTW 3 documents it), computed
// here with direct discrete Fourier transforms in double along each axis, so
// that the reference's bilateral tone mapper (camera.cc:1632-1812) runs.
// Conventions of FFTW: arrays row-major over the dimensions as given (the
// last varies fastest); forward transforms use exp(-2 pi i j k / n), backward
// exp(+2 pi i j k / n), neither normalised; a real-to-complex transform
// stores the non-negative half of the last dimension (n_last / 2 + 1
// entries), a complex-to-real one reads that half and assumes Hermitian
// symmetry for the rest.  howmany transforms follow at idist / odist
// elements (unit strides, no embedding, which is all the reference asks).
// The results differ from FFTW's by FFTW's own single-precision rounding.
}  // extern "C"

#include <cmath>
#include <complex>
#include <vector>

namespace {

using cd = std::complex<double>;

enum Kind { kC2C, kR2C, kC2R };

struct Plan {
    Kind kind;
    std::vector<int> n;
    int howmany;
    int idist, odist;
    void *in, *out;
    int sign;
};

// In-place DFT of a full complex array (dims n, row-major) along every axis.
void dft_all(std::vector<cd> &a, const std::vector<int> &n, int sign)
{
    const int rank = (int)n.size();
    size_t total = 1;
    for (int v : n) total *= (size_t)v;
    std::vector<cd> line, res;
    for (int ax = 0; ax < rank; ++ax) {
        const int m = n[(size_t)ax];
        size_t inner = 1;
        for (int k = ax + 1; k < rank; ++k) inner *= (size_t)n[(size_t)k];
        const size_t outer = total / ((size_t)m * inner);
        std::vector<cd> tw((size_t)m);
        for (int k = 0; k < m; ++k) {
            const double ang = 2.0 * M_PI * (double)k / (double)m;
            tw[(size_t)k] = cd(std::cos(ang), (double)sign * std::sin(ang));
        }
        line.resize((size_t)m);
        res.resize((size_t)m);
        for (size_t o = 0; o < outer; ++o)
            for (size_t in = 0; in < inner; ++in) {
                const size_t base = o * (size_t)m * inner + in;
                for (int j = 0; j < m; ++j) line[(size_t)j] = a[base + (size_t)j * inner];
                for (int k = 0; k < m; ++k) {
                    cd acc(0.0, 0.0);
                    for (int j = 0; j < m; ++j) acc += line[(size_t)j] * tw[(size_t)(((long long)j * k) % m)];
                    res[(size_t)k] = acc;
                }
                for (int k = 0; k < m; ++k) a[base + (size_t)k * inner] = res[(size_t)k];
            }
    }
}

size_t count(const std::vector<int> &n)
{
    size_t t = 1;
    for (int v : n) t *= (size_t)v;
    return t;
}

// Index of the Hermitian partner of full-array index idx (every coordinate
// negated modulo its dimension).
size_t mirror(size_t idx, const std::vector<int> &n)
{
    const int rank = (int)n.size();
    std::vector<int> c((size_t)rank);
    for (int ax = rank - 1; ax >= 0; --ax) {
        c[(size_t)ax] = (int)(idx % (size_t)n[(size_t)ax]);
        idx /= (size_t)n[(size_t)ax];
    }
    size_t r = 0;
    for (int ax = 0; ax < rank; ++ax) {
        const int m = n[(size_t)ax];
        r = r * (size_t)m + (size_t)((m - c[(size_t)ax]) % m);
    }
    return r;
}

void run(const Plan &P)
{
    const size_t total = count(P.n);
    const int last = P.n.back();
    const int half = last / 2 + 1;
    const size_t rows = total / (size_t)last;
    std::vector<cd> a(total);
    for (int h = 0; h < P.howmany; ++h) {
        if (P.kind == kC2C) {
            const float(*in)[2] = reinterpret_cast<const float(*)[2]>(P.in) + (size_t)h * (size_t)P.idist;
            for (size_t i = 0; i < total; ++i) a[i] = cd(in[i][0], in[i][1]);
            dft_all(a, P.n, P.sign);
            float(*out)[2] = reinterpret_cast<float(*)[2]>(P.out) + (size_t)h * (size_t)P.odist;
            for (size_t i = 0; i < total; ++i) { out[i][0] = (float)a[i].real(); out[i][1] = (float)a[i].imag(); }
        } else if (P.kind == kR2C) {
            const float *in = reinterpret_cast<const float *>(P.in) + (size_t)h * (size_t)P.idist;
            for (size_t i = 0; i < total; ++i) a[i] = cd(in[i], 0.0);
            dft_all(a, P.n, -1);
            float(*out)[2] = reinterpret_cast<float(*)[2]>(P.out) + (size_t)h * (size_t)P.odist;
            for (size_t r = 0; r < rows; ++r)
                for (int k = 0; k < half; ++k) {
                    const cd v = a[r * (size_t)last + (size_t)k];
                    out[r * (size_t)half + (size_t)k][0] = (float)v.real();
                    out[r * (size_t)half + (size_t)k][1] = (float)v.imag();
                }
        } else {
            const float(*in)[2] = reinterpret_cast<const float(*)[2]>(P.in) + (size_t)h * (size_t)P.idist;
            for (size_t r = 0; r < rows; ++r)
                for (int k = 0; k < half; ++k)
                    a[r * (size_t)last + (size_t)k] = cd(in[r * (size_t)half + (size_t)k][0],
                                                         in[r * (size_t)half + (size_t)k][1]);
            for (size_t i = 0; i < total; ++i)
                if ((int)(i % (size_t)last) >= half) a[i] = std::conj(a[mirror(i, P.n)]);
            dft_all(a, P.n, +1);
            float *out = reinterpret_cast<float *>(P.out) + (size_t)h * (size_t)P.odist;
            for (size_t i = 0; i < total; ++i) out[i] = (float)a[i].real();
        }
    }
}

fftwf_plan make(Kind k, int rank, const int *n, int howmany, void *in, int idist, void *out, int odist, int sign)
{
    Plan *p = new Plan;
    p->kind = k;
    p->n.assign(n, n + rank);
    p->howmany = howmany;
    p->idist = idist;
    p->odist = odist;
    p->in = in;
    p->out = out;
    p->sign = sign;
    return reinterpret_cast<fftwf_plan>(p);
}

}  // namespace

extern "C" {
void *fftwf_malloc(size_t n) { return std::malloc(n ? n : 1); }
void fftwf_free(void *p) { std::free(p); }
void fftwf_execute(const fftwf_plan p) { run(*reinterpret_cast<const Plan *>(p)); }
void fftwf_destroy_plan(fftwf_plan p) { delete reinterpret_cast<Plan *>(p); }
fftwf_plan fftwf_plan_dft_2d(int n0, int n1, fftwf_complex *in, fftwf_complex *out, int sign, unsigned)
{
    const int n[2] = {n0, n1};
    return make(kC2C, 2, n, 1, in, 0, out, 0, sign);
}
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *out, unsigned)
{
    const int n[3] = {n0, n1, n2};
    return make(kR2C, 3, n, 1, in, 0, out, 0, -1);
}
fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany, float *in, const int *, int, int idist,
                                   fftwf_complex *out, const int *, int, int odist, unsigned)
{
    return make(kR2C, rank, n, howmany, in, idist, out, odist, -1);
}
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany, fftwf_complex *in, const int *, int, int idist,
                                   float *out, const int *, int, int odist, unsigned)
{
    return make(kC2R, rank, n, howmany, in, idist, out, odist, +1);
}
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

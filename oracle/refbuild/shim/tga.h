// Declaration-only stand-in for libtga. The reference's inline image readers
// reference these names; they are never called on the traced path.
#pragma once
#include <cstdio>
typedef unsigned char tbyte;
typedef unsigned short tshort;
typedef unsigned int tuint;
typedef unsigned int tlong;
#define TGA_OK 0
#define TGA_IMAGE_DATA 1
#define TGA_COLOR_MAP 2
#define TGA_IMAGE_ID 4
#define TGA_RGB 8
#define TGA_BGR 16
#define TGA_RLE_ENCODE 32
#define TGA_IMAGE_INFO 64
#define TGA_RGB24 2
struct TGAHeader { tbyte id_len, map_t, img_t; tshort map_first, map_len; tbyte map_entry; tshort x, y, width, height; tbyte depth, alpha, horz, vert; };
struct TGA { FILE *fd; tlong off; int last; TGAHeader hdr; };
struct TGAData { tbyte *img_id; tbyte *cmap; tbyte *img_data; tuint flags; };
TGA *TGAOpen(char *, const char *);
int TGAReadImage(TGA *, TGAData *);
int TGAWriteImage(TGA *, TGAData *);
void TGAClose(TGA *);

// rt_mesh_io.cpp -- scene ingest: OFF and PLY meshes read into the indexed
// arrays rt_scene_upload takes, with the triangles (and their order) the
// reference's parsers put into its primitive_store, so triangle ids match.
//
// Reference behaviour restated (RAPTor paths):
//   raytracer/parsers/off_parser.cc   header "OFF", counts, vertices, faces;
//                                     3-vertex faces kept as they are, larger
//                                     faces triangulated, default diffuse 170
//   raytracer/parsers/ply_parser.cc   "format ascii 1.0" or
//                                     "format binary_big_endian 1.0"; vertex
//                                     x y z (+ optional uchar colour and float
//                                     normal, parsed and not used), faces as
//                                     uchar count + int indices (+ optional
//                                     leading uchar intensity, trailing uchar
//                                     colour); degenerate triangles dropped;
//                                     default diffuse 200, face colours in
//                                     binary files
//   raytracer/parsers/obj_parser.cc   v / vt / vn / f (v, v/t, v//n, v/t/n,
//                                     negative indices relative to the end),
//                                     usemtl groups, g / o / s and comments
//                                     skipped, degenerate triangles dropped;
//                                     material libraries are not read
//   raytracer/parsers/polygon_to_triangles.h  the ear-clipping of faces with
//                                     more than 3 vertices (face_to_triangles)
//   parsers/parser_common.h           token rules: numbers read by atof/atoi
//                                     after the reference's own skipping of
//                                     spaces, tabs and separators
// Host code only (no device work): it feeds rt_scene_upload.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "rtcore.h"

rt_status rt_set_error_message(rt_status code, const char *msg);

namespace {

struct V3 {
    float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 cross(V3 a, V3 b) { return {(a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x)}; }
float dot(V3 a, V3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
float mag(V3 a) { return std::sqrt(((a.x * a.x) + (a.y * a.y)) + (a.z * a.z)); }
V3 unit(V3 a)
{
    const float d = mag(a);
    return {a.x / d, a.y / d, a.z / d};
}
bool all_zero(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
bool differ(V3 a, V3 b) { return a.x != b.x || a.y != b.y || a.z != b.z; }

struct Mesh {
    std::vector<float> verts;
    std::vector<int32_t> tris;
    std::vector<uint8_t> rgb;   // per triangle, when the file colours its faces
    std::vector<int32_t> mat;   // per triangle, when the file names materials
    std::vector<float> cn;      // 9 per triangle (corner normals), when the file has vertex normals
    bool coloured = false, named = false, normals = false;
    int32_t cur_mat = 0, nmat = 1;
    float kd = 0.0f;
    V3 vert(int32_t i) const { return {verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]}; }
    void add(int32_t a, int32_t b, int32_t c, const uint8_t *col, const V3 *nrm = nullptr)
    {
        tris.push_back(a);
        tris.push_back(b);
        tris.push_back(c);
        if (coloured) rgb.insert(rgb.end(), col, col + 3);
        if (named) mat.push_back(cur_mat);
        if (normals) {
            for (int k = 0; k < 3; ++k) {
                cn.push_back(nrm ? nrm[k].x : 3.402823466e38f);
                cn.push_back(nrm ? nrm[k].y : 0.0f);
                cn.push_back(nrm ? nrm[k].z : 0.0f);
            }
        }
    }
};

// Ear clipping of one face (indices into the mesh's vertices), in the order
// polygon_to_triangles.h's face_to_triangles emits triangles: start at the
// vertex furthest from the face's centroid, take the face normal from its
// two neighbours, and walk the ring accepting (prev, cur, next) when it turns
// the face's way and holds no face vertex strictly inside; a collinear
// triple drops its middle vertex without a triangle; stop when two vertices
// remain or a full lap accepts nothing.
void triangulate(Mesh &m, const std::vector<int32_t> &face, const uint8_t *col,
                 const std::vector<V3> *fnorm = nullptr)
{
    const size_t n = face.size();
    if (n < 3) return;
    std::vector<V3> p(n);
    for (size_t i = 0; i < n; ++i) p[i] = m.vert(face[i]);
    V3 centre = {0.0f, 0.0f, 0.0f};
    for (const V3 &q : p) centre = {centre.x + q.x, centre.y + q.y, centre.z + q.z};
    const float cnt = (float)n;
    centre = {centre.x / cnt, centre.y / cnt, centre.z / cnt};
    size_t cur = 0;
    float far = 0.0f;
    for (size_t i = 0; i < n; ++i) {
        const float d = mag(sub(centre, p[i]));
        if (d > far) {
            far = d;
            cur = i;
        }
    }
    size_t prev = (cur == 0) ? n - 1 : cur - 1;
    size_t next = (cur == n - 1) ? 0 : cur + 1;
    const V3 fn = unit(cross(sub(p[prev], p[cur]), sub(p[cur], p[next])));
    // same side of edge (a, a + ab) as the face normal, strictly
    auto same_side = [&](V3 q, V3 a, V3 ab) { return dot(cross(sub(q, a), ab), fn) > 0.0f; };
    std::vector<char> gone(n, 0);
    size_t left = n, misses = 0;
    for (size_t guard = 0; guard < 4 * n * n + 16; ++guard) {
        bool accepted = true;
        const V3 a = p[prev], b = p[cur], c = p[next];
        if (!all_zero(cross(sub(b, a), sub(c, a)))) {
            const V3 tn = unit(cross(sub(a, b), sub(b, c)));
            bool inside = false;
            if (dot(tn, fn) > 0.0f) {
                const V3 ab = sub(a, b), ca = sub(c, a), bc = sub(b, c);
                for (size_t i = 0; i < n && !inside; ++i)
                    inside = same_side(p[i], a, ab) && same_side(p[i], b, bc) && same_side(p[i], c, ca);
            }
            if (dot(tn, fn) > 0.0f && !inside) {
                if (fnorm) {
                    const V3 cn3[3] = {(*fnorm)[prev], (*fnorm)[cur], (*fnorm)[next]};
                    m.add(face[prev], face[cur], face[next], col, cn3);
                } else {
                    m.add(face[prev], face[cur], face[next], col);
                }
            } else {
                accepted = false;
            }
        }
        if (accepted) {
            --left;
            misses = 0;
            gone[cur] = 1;
        } else {
            prev = cur;
            ++misses;
        }
        cur = next;
        do {
            ++next;
            if (next == n) next = 0;
        } while (gone[next]);
        if (left == 2 || misses == left) break;
    }
}

// Token rules of the reference's byte-stream parser (parser_common.h).
struct Cursor {
    const char *c, *end;
    void skip_blanks()   // spaces and tabs
    {
        while (c < end && (*c == ' ' || *c == '\t')) ++c;
    }
    void skip_spaces()
    {
        while (c < end && *c == ' ') ++c;
    }
    // atof / atoi on a bounded copy of the token at c (leading white space
    // skipped as they skip it; the number ends at a separator at the latest)
    size_t token(char *buf, size_t cap) const
    {
        size_t k = 0;
        const char *q = c;
        while (q < end && (*q == ' ' || *q == '\t' || *q == '\r' || *q == '\n')) ++q;
        while (q < end && k < cap - 1 && !(*q == ' ' || *q == '\t' || *q == '\r' || *q == '\n' || *q == '/'))
            buf[k++] = *q++;
        buf[k] = '\0';
        return k;
    }
    double number_here() const
    {
        char buf[512];
        token(buf, sizeof(buf));
        return std::strtod(buf, nullptr);
    }
    long int_here() const
    {
        char buf[64];
        token(buf, sizeof(buf));
        return std::strtol(buf, nullptr, 10);
    }
    float this_float()
    {
        skip_blanks();
        return (float)number_here();
    }
    float next_float()   // past the current token and the blanks after it
    {
        while (c < end && *c != ' ' && *c != '\t') ++c;
        skip_blanks();
        return (float)number_here();
    }
    long this_int()
    {
        skip_spaces();
        return int_here();
    }
    long next_int()   // past the current token, one separator and spaces
    {
        while (c < end && *c != ' ' && *c != '/') ++c;
        if (c < end) ++c;
        skip_spaces();
        return int_here();
    }
    std::string this_word()
    {
        skip_spaces();
        const char *s = c;
        while (c < end && *c != ' ' && *c != '\n') ++c;
        return std::string(s, c);
    }
    bool next_line()   // past the current character, then past the next newline
    {
        if (c < end) ++c;
        while (c < end && *c != '\n') ++c;
        if (c < end) {
            ++c;
            return true;
        }
        return false;
    }
    bool starts(const char *s) const
    {
        const size_t n = std::strlen(s);
        return (size_t)(end - c) >= n && std::strncmp(c, s, n) == 0;
    }
};

rt_status bad(const char *msg) { return rt_set_error_message(RT_ERR_INVALID_ARG, msg); }

rt_status parse_off(Cursor cur, Mesh &m)
{
    m.kd = 170.0f;
    const std::string head = cur.this_word();
    if (head != "OFF" && head != "OFF\r") return bad("rt_mesh: not an OFF file");
    const long nv = cur.this_int();
    const long nf = cur.next_int();
    cur.next_int();   // edges
    cur.next_line();
    if (nv < 0 || nf < 0 || nv > (1l << 28) || nf > (1l << 28)) return bad("rt_mesh: OFF counts out of range");
    m.verts.reserve(3 * nv);
    for (long i = 0; i < nv; ++i) {
        if (cur.c >= cur.end) return bad("rt_mesh: OFF file ends inside the vertex list");
        m.verts.push_back(cur.this_float());
        m.verts.push_back(cur.next_float());
        m.verts.push_back(cur.next_float());
        cur.next_line();
    }
    std::vector<int32_t> face;
    for (long i = 0; i < nf; ++i) {
        if (cur.c >= cur.end) return bad("rt_mesh: OFF file ends inside the face list");
        const long k = cur.this_int();
        if (k < 0 || k > (1l << 20)) return bad("rt_mesh: OFF face size out of range");
        face.clear();
        for (long j = 0; j < k; ++j) {
            const long idx = cur.next_int();
            if (idx < 0 || idx >= nv) return bad("rt_mesh: OFF vertex index out of range");
            face.push_back((int32_t)idx);
        }
        cur.next_line();
        if (face.size() == 3) m.add(face[0], face[1], face[2], nullptr);
        else if (face.size() > 3) triangulate(m, face, nullptr);
    }
    return RT_OK;
}

// ply_parser.cc: the next header statement, skipping comment / obj_info lines.
void ply_next(Cursor &cur)
{
    do {
        if (!cur.next_line()) return;
    } while (cur.starts("comment ") || cur.starts("obj_info "));
}

rt_status parse_ply(Cursor cur, Mesh &m)
{
    m.kd = 200.0f;
    if (!cur.starts("ply")) return bad("rt_mesh: not a PLY file");
    ply_next(cur);
    bool binary;
    if (cur.starts("format ascii 1.0")) binary = false;
    else if (cur.starts("format binary_big_endian 1.0")) binary = true;
    else return bad("rt_mesh: PLY format must be ascii 1.0 or binary_big_endian 1.0");
    ply_next(cur);
    // vertex element
    if (!cur.starts("element vertex ")) return bad("rt_mesh: PLY header lacks 'element vertex'");
    cur.c += 14;
    const long nv = cur.next_int();
    const char *axes[3][2] = {{"property float x", "property float32 x"}, {"property float y", "property float32 y"},
                              {"property float z", "property float32 z"}};
    for (int a = 0; a < 3; ++a) {
        ply_next(cur);
        if (!cur.starts(axes[a][0]) && !cur.starts(axes[a][1]))
            return bad("rt_mesh: PLY vertices must start with float x, y, z");
    }
    ply_next(cur);
    unsigned v_skip = 0;
    bool v_colour = false, v_normal = false;
    while (cur.starts("property ")) {
        if (cur.starts("property uchar red")) {
            ply_next(cur);
            if (cur.starts("property uchar green")) {
                ply_next(cur);
                if (cur.starts("property uchar blue")) {
                    v_colour = true;
                    ply_next(cur);
                } else {
                    v_skip += 2;
                }
            } else {
                v_skip += 1;
            }
            if (!cur.starts("property ")) break;
        }
        if (cur.starts("property float nx")) {
            ply_next(cur);
            if (cur.starts("property float ny")) {
                ply_next(cur);
                if (cur.starts("property float nz")) {
                    v_normal = true;
                    ply_next(cur);
                } else {
                    v_skip += 2;
                }
            } else {
                v_skip += 1;
            }
            if (!cur.starts("property ")) break;
        }
        if (std::strncmp(cur.c + 9, "uchar ", 6) == 0 || std::strncmp(cur.c + 9, "uint8 ", 6) == 0) v_skip += 1;
        else if (std::strncmp(cur.c + 9, "float ", 6) == 0 || std::strncmp(cur.c + 9, "float32 ", 8) == 0) v_skip += 4;
        else return bad("rt_mesh: unsupported PLY vertex property");
        ply_next(cur);
    }
    // face element
    if (!cur.starts("element face ")) return bad("rt_mesh: PLY header lacks 'element face'");
    cur.c += 12;
    const long nf = cur.next_int();
    ply_next(cur);
    unsigned pre_skip = 0, post_skip = 0;
    bool f_colour = false;
    if (cur.starts("property uchar intensity")) {
        pre_skip = 1;
        ply_next(cur);
    }
    if (!cur.starts("property list uchar int vertex_indices") && !cur.starts("property list uint8 int32 vertex_indices"))
        return bad("rt_mesh: PLY faces must be 'property list uchar int vertex_indices'");
    ply_next(cur);
    while (cur.starts("property ")) {
        if (cur.starts("property uchar red")) {
            ply_next(cur);
            if (cur.starts("property uchar green")) {
                ply_next(cur);
                if (cur.starts("property uchar blue")) {
                    f_colour = true;
                    ply_next(cur);
                } else {
                    post_skip += 2;
                }
            } else {
                post_skip += 1;
            }
            if (!cur.starts("property ")) break;
        }
        if (std::strncmp(cur.c + 9, "uchar ", 6) == 0 || std::strncmp(cur.c + 9, "uint8 ", 6) == 0) post_skip += 1;
        else return bad("rt_mesh: unsupported PLY face property");
        ply_next(cur);
    }
    if (!cur.starts("end_header")) return bad("rt_mesh: PLY header lacks 'end_header'");
    ply_next(cur);
    if (nv < 0 || nf < 0 || nv > (1l << 28) || nf > (1l << 28)) return bad("rt_mesh: PLY counts out of range");
    if (!binary && f_colour) return bad("rt_mesh: face colours in ascii PLY are not supported");
    m.coloured = f_colour;
    m.verts.reserve(3 * nv);
    auto be32 = [&](uint32_t &out) {
        if (cur.end - cur.c < 4) return false;
        const unsigned char *b = (const unsigned char *)cur.c;
        out = ((uint32_t)b[0] << 24) | ((uint32_t)b[1] << 16) | ((uint32_t)b[2] << 8) | (uint32_t)b[3];
        cur.c += 4;
        return true;
    };
    for (long i = 0; i < nv; ++i) {
        if (binary) {
            for (int a = 0; a < 3; ++a) {
                uint32_t w;
                if (!be32(w)) return bad("rt_mesh: PLY file ends inside the vertex list");
                float f;
                std::memcpy(&f, &w, 4);
                m.verts.push_back(f);
            }
            const long extra = (v_colour ? 3 : 0) + (v_normal ? 12 : 0) + v_skip;
            if (cur.end - cur.c < extra) return bad("rt_mesh: PLY file ends inside the vertex list");
            cur.c += extra;
        } else {
            if (cur.c >= cur.end) return bad("rt_mesh: PLY file ends inside the vertex list");
            m.verts.push_back((float)cur.number_here());
            m.verts.push_back(cur.next_float());
            m.verts.push_back(cur.next_float());
            if (v_normal) {
                cur.next_float();
                cur.next_float();
                cur.next_float();
            }
            cur.next_line();
        }
    }
    std::vector<int32_t> face;
    uint8_t col[3] = {0, 0, 0};
    for (long i = 0; i < nf; ++i) {
        if (cur.c >= cur.end) return bad("rt_mesh: PLY file ends inside the face list");
        cur.c += pre_skip;
        face.clear();
        if (binary) {
            if (cur.c >= cur.end) return bad("rt_mesh: PLY file ends inside the face list");
            const unsigned k = (unsigned char)*cur.c++;
            for (unsigned j = 0; j < k; ++j) {
                uint32_t w;
                if (!be32(w)) return bad("rt_mesh: PLY file ends inside the face list");
                const int32_t idx = (int32_t)w;
                if (idx < 0 || idx >= nv) return bad("rt_mesh: PLY vertex index out of range");
                face.push_back(idx);
            }
            if (f_colour) {
                if (cur.end - cur.c < 3) return bad("rt_mesh: PLY file ends inside the face list");
                std::memcpy(col, cur.c, 3);
                cur.c += 3;
            }
        } else {
            const long k = cur.int_here();
            if (k < 0 || k > (1l << 20)) return bad("rt_mesh: PLY face size out of range");
            for (long j = 0; j < k; ++j) {
                const long idx = cur.next_int();
                if (idx < 0 || idx >= nv) return bad("rt_mesh: PLY vertex index out of range");
                face.push_back((int32_t)idx);
            }
            cur.next_line();
        }
        if (face.size() == 3) {
            // ply_parser.cc drops triangles whose points do not move in at
            // least two axes (two equal points, or parallel unit edges)
            const V3 a0 = m.vert(face[0]), b0 = m.vert(face[1]), c0 = m.vert(face[2]);
            if (differ(a0, b0) && differ(a0, c0) && differ(b0, c0)) {
                const V3 ea = unit(sub(a0, b0)), eb = unit(sub(b0, c0));
                const V3 d = sub(ea, eb), s = {ea.x + eb.x, ea.y + eb.y, ea.z + eb.z};
                if (!all_zero(d) && !all_zero(s)) m.add(face[0], face[1], face[2], col);
            }
        } else {
            triangulate(m, face, col);
        }
        if (binary) cur.c += post_skip;
    }
    return RT_OK;
}

// obj_parser.cc: the next statement, past white space and '#' comments.
const char *obj_statement(const char *at, const char *end)
{
    while (at < end) {
        if (*at == '#') {
            while (at < end && *at != '\n') ++at;
            ++at;
        } else if (*at == ' ' || *at == '\t' || *at == '\n' || *at == '\r') {
            ++at;
        } else {
            return at;
        }
    }
    return end;
}

rt_status parse_obj(Cursor cur, Mesh &m)
{
    m.kd = 200.0f;
    m.named = true;
    std::vector<std::string> names;   // usemtl names in order of first use (index + 1)
    long nvt = 0, nvn = 0;
    std::vector<V3> vn;                // unit vertex normals (parse_vn_statement normalises)
    std::vector<int32_t> face;
    std::vector<V3> face_n;
    const char *const last = cur.end - 1;   // the reference stops one byte before the end
    while (cur.c < last) {
        cur.c = obj_statement(cur.c, last);
        if (cur.c >= last) break;
        if (cur.starts("mtllib")) {
            cur.next_line();   // material libraries are not read
        } else if (cur.starts("usemtl")) {
            // raptor_parsers::get_next_string: the word after the keyword
            while (cur.c < cur.end && *cur.c != ' ') ++cur.c;
            cur.skip_spaces();
            const char *s = cur.c;
            while (cur.c < cur.end && *cur.c != ' ' && *cur.c != '\n' && *cur.c != '\r') ++cur.c;
            const std::string name(s, cur.c);
            size_t k = 0;
            while (k < names.size() && names[k] != name) ++k;
            if (k == names.size()) names.push_back(name);
            m.cur_mat = (int32_t)k + 1;
            --cur.c;
            cur.next_line();
        } else if (cur.starts("vn")) {
            V3 n;
            n.x = cur.next_float();
            n.y = cur.next_float();
            n.z = cur.next_float();
            cur.next_line();
            vn.push_back(unit(n));
            m.normals = true;
            ++nvn;
        } else if (cur.starts("vt")) {
            cur.next_float();
            cur.next_float();
            cur.next_line();
            ++nvt;
        } else if (*cur.c == 'f') {
            // find_vertex: past the keyword, then spaces
            auto find_vertex = [&]() {
                while (cur.c < cur.end && *cur.c != ' ' && *cur.c != '\n' && *cur.c != '\r') ++cur.c;
                cur.skip_spaces();
            };
            // is_triplet_delimiter: past one character, then to '/' or the field's end
            auto delimiter = [&]() {
                ++cur.c;
                while (cur.c < cur.end && *cur.c != '/' && *cur.c != ' ' && *cur.c != '\n' && *cur.c != '\r') ++cur.c;
                return cur.c < cur.end && *cur.c == '/';
            };
            const long nv = (long)(m.verts.size() / 3);
            face.clear();
            face_n.clear();
            find_vertex();
            while (cur.c < cur.end && *cur.c != '\n' && *cur.c != '\r') {
                long vi = std::strtol(cur.c, nullptr, 10);
                vi = (vi < 0) ? nv + vi : vi - 1;
                if (vi < 0 || vi >= nv) return bad("rt_mesh: OBJ vertex index out of range");
                face.push_back((int32_t)vi);
                if (delimiter()) {
                    if (cur.c + 1 < cur.end && cur.c[1] != '/') {
                        ++cur.c;
                        long ti = std::strtol(cur.c, nullptr, 10);
                        ti = (ti < 0) ? nvt + ti : ti - 1;
                        if (ti < 0 || ti >= nvt) return bad("rt_mesh: OBJ texture index out of range");
                    }
                    if (delimiter()) {
                        ++cur.c;
                        long ni = std::strtol(cur.c, nullptr, 10);
                        ni = (ni < 0) ? nvn + ni : ni - 1;
                        if (ni < 0 || ni >= nvn) return bad("rt_mesh: OBJ normal index out of range");
                        face_n.push_back(vn[ni]);
                    }
                }
                find_vertex();
            }
            if (cur.c < cur.end) ++cur.c;
            if (face.size() == 3) {
                // obj_parser.cc drops triangles with two equal points or
                // parallel unit edges (zero cross product)
                const V3 a0 = m.vert(face[0]), b0 = m.vert(face[1]), c0 = m.vert(face[2]);
                if (differ(a0, b0) && differ(a0, c0) && differ(b0, c0)) {
                    const V3 n = cross(unit(sub(a0, b0)), unit(sub(b0, c0)));
                    if (dot(n, n) > 0.0f)
                        m.add(face[0], face[1], face[2], nullptr, face_n.size() == 3 ? face_n.data() : nullptr);
                }
            } else {
                triangulate(m, face, nullptr, face_n.size() == face.size() ? &face_n : nullptr);
            }
        } else if (*cur.c == 'v') {
            m.verts.push_back(cur.next_float());
            m.verts.push_back(cur.next_float());
            m.verts.push_back(cur.next_float());
            cur.next_line();
        } else {
            // g, o, s and statements the reference does not know: the line is skipped
            cur.next_line();
        }
    }
    m.nmat = (int32_t)names.size() + 1;
    return RT_OK;
}

bool ends_with(const std::string &s, const char *suf)
{
    const size_t n = std::strlen(suf);
    if (s.size() < n) return false;
    for (size_t i = 0; i < n; ++i)
        if (std::tolower((unsigned char)s[s.size() - n + i]) != suf[i]) return false;
    return true;
}

template <typename T> T *copy_out(const std::vector<T> &v)
{
    T *p = (T *)std::malloc(v.empty() ? sizeof(T) : v.size() * sizeof(T));
    if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" {

rt_status rt_mesh_parse(const char *data, int64_t len, int32_t format, rt_mesh *out)
{
    if (!data || !out || len < 0) return bad("rt_mesh_parse: NULL argument");
    std::memset(out, 0, sizeof(*out));
    if (format != RT_MESH_OFF && format != RT_MESH_PLY && format != RT_MESH_OBJ)
        return bad("rt_mesh_parse: format must be RT_MESH_OFF, PLY or OBJ");
    // a NUL-terminated copy: the token rules read up to the next separator
    std::vector<char> buf((size_t)len + 1, '\0');
    std::memcpy(buf.data(), data, (size_t)len);
    Cursor cur{buf.data(), buf.data() + len};
    Mesh m;
    rt_status st;
    try {
        st = (format == RT_MESH_OFF) ? parse_off(cur, m) : (format == RT_MESH_PLY) ? parse_ply(cur, m) : parse_obj(cur, m);
    } catch (const std::bad_alloc &) {
        return rt_set_error_message(RT_ERR_OUT_OF_MEMORY, "rt_mesh_parse: out of host memory");
    }
    if (st != RT_OK) return st;
    out->nverts = (int32_t)(m.verts.size() / 3);
    out->ntris = (int32_t)(m.tris.size() / 3);
    out->verts = copy_out(m.verts);
    out->tris = copy_out(m.tris);
    out->tri_rgb = m.coloured ? copy_out(m.rgb) : nullptr;
    out->tri_mat = m.named ? copy_out(m.mat) : nullptr;
    out->corner_normals = m.normals ? copy_out(m.cn) : nullptr;
    out->nmat = m.nmat;
    out->kd[0] = out->kd[1] = out->kd[2] = m.kd;
    if (!out->verts || !out->tris || (m.coloured && !out->tri_rgb) || (m.named && !out->tri_mat) ||
        (m.normals && !out->corner_normals)) {
        rt_mesh_free(out);
        return rt_set_error_message(RT_ERR_OUT_OF_MEMORY, "rt_mesh_parse: out of host memory");
    }
    return RT_OK;
}

rt_status rt_mesh_load(const char *path, int32_t format, rt_mesh *out)
{
    if (!path || !out) return bad("rt_mesh_load: NULL argument");
    std::memset(out, 0, sizeof(*out));
    if (format == RT_MESH_AUTO) {
        const std::string p(path);
        if (ends_with(p, ".off")) format = RT_MESH_OFF;
        else if (ends_with(p, ".ply")) format = RT_MESH_PLY;
        else if (ends_with(p, ".obj")) format = RT_MESH_OBJ;
        else return bad("rt_mesh_load: unknown file extension (expected .off, .ply or .obj)");
    }
    FILE *f = std::fopen(path, "rb");
    if (!f) return bad("rt_mesh_load: cannot open the file");
    std::vector<char> data;
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) data.insert(data.end(), chunk, chunk + got);
    std::fclose(f);
    return rt_mesh_parse(data.data(), (int64_t)data.size(), format, out);
}

void rt_mesh_free(rt_mesh *m)
{
    if (!m) return;
    std::free(m->verts);
    std::free(m->tris);
    std::free(m->tri_rgb);
    std::free(m->tri_mat);
    std::free(m->corner_normals);
    m->corner_normals = nullptr;
    m->verts = nullptr;
    m->tris = nullptr;
    m->tri_rgb = nullptr;
    m->tri_mat = nullptr;
    m->nverts = m->ntris = 0;
}

}  // extern "C"

// mesh_io.cpp -- TetGen mesh ingest (host only): the reference's converter
// examples/tetgen2geo/main.cpp restated for fem_solid_create's inputs.
//
// What follows the converter:
//   .node: "num_nodes dim num_attrib num_boundary", then per node
//          "vid x y z [attrib...] [marker]"; the first vid is the base index
//          of every id (0 or 1 in TetGen output; the converter's base_vid),
//          positions read as float (its Vec3f), attributes and markers skipped;
//   .ele:  "num_tets nodes_per_tet num_attrib", then per tet
//          "tid v0 v1 v2 v3 [attrib...]", ids made base-0 by base_vid;
//   tets whose det(x1-x0, x2-x0, x3-x0) <= 0 in float are dropped, as
//   EditableTetSolidShape3::AddTetrahedron ignores them
//   (Geo/shape/TetSolidShape3.cpp:278-307);
//   the optional natural scale ("-nsac s"): the float AABB of the nodes,
//   merged node by node as GAABB::Merge does (Geo/bv/GAABB.h:27-50), then
//   positions moved by -center and scaled by s / max(2 half_sizes).
// The .face file is not read (the converter reads it but no longer uses it).
// The shape the converter then builds (EndEdition's rebuild) and the
// shape-library file it writes are in shape_io.cpp.
#include "../../include/fem_tet.h"

#include <cctype>
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace femgb {
void set_last_error(const char* msg);
}

namespace {

int io_fail(int code, const std::string& msg)
{
    femgb::set_last_error(msg.c_str());
    return code;
}

// Whitespace-separated tokens; '#' starts a comment to the end of the line
// (TetGen writes its comments at the end of its files).
class Tokens {
public:
    explicit Tokens(FILE* f) : f_(f) {}
    bool next(std::string& tok)
    {
        tok.clear();
        int c;
        for (;;) {
            c = std::fgetc(f_);
            if (c == EOF) return false;
            if (c == '#') {
                while (c != EOF && c != '\n') c = std::fgetc(f_);
                continue;
            }
            if (!std::isspace(c)) break;
        }
        while (c != EOF && !std::isspace(c) && c != '#') {
            tok.push_back((char)c);
            c = std::fgetc(f_);
        }
        if (c == '#') std::ungetc(c, f_);
        return true;
    }
    bool next_long(long& v)
    {
        std::string t;
        if (!next(t)) return false;
        char* end = nullptr;
        errno = 0;
        v = std::strtol(t.c_str(), &end, 10);
        return errno == 0 && end && *end == '\0';
    }
    bool next_float(float& v)
    {
        std::string t;
        if (!next(t)) return false;
        char* end = nullptr;
        errno = 0;
        v = std::strtof(t.c_str(), &end);
        return end && *end == '\0' && end != t.c_str();
    }

private:
    FILE* f_;
};

struct File {
    FILE* f = nullptr;
    ~File()
    {
        if (f) std::fclose(f);
    }
};

// mal::Det of the float matrix with columns (a, b, c) (Mal/GMat.h:236-245)
float det_columns(const float* a, const float* b, const float* c)
{
    // m(i, j): column j; row-major m[3 i + j] = col_j[i]
    const float m[9] = {a[0], b[0], c[0], a[1], b[1], c[1], a[2], b[2], c[2]};
    return m[0] * m[4] * m[8] - m[0] * m[7] * m[5] + m[3] * m[7] * m[2] - m[3] * m[1] * m[8] + m[6] * m[1] * m[5] -
           m[6] * m[4] * m[2];
}

}  // namespace

namespace {
int tetgen_read(const char* node_path, const char* ele_path, double natural_scale, double* rest, uint32_t max_nodes,
                uint32_t* tets, uint32_t max_tets, uint32_t* num_nodes, uint32_t* num_tets, uint32_t* num_dropped);
}

// No C++ exception leaves the C ABI: a header whose counts do not fit in host
// memory answers FEM_E_OOM.
extern "C" int fem_tetgen_read(const char* node_path, const char* ele_path, double natural_scale, double* rest,
                               uint32_t max_nodes, uint32_t* tets, uint32_t max_tets, uint32_t* num_nodes,
                               uint32_t* num_tets, uint32_t* num_dropped)
{
    try {
        return tetgen_read(node_path, ele_path, natural_scale, rest, max_nodes, tets, max_tets, num_nodes, num_tets,
                           num_dropped);
    } catch (const std::bad_alloc&) {
        return io_fail(FEM_E_OOM, "host allocation failed while reading the mesh");
    } catch (...) {
        return io_fail(FEM_E_ARG, "failed to read the mesh");
    }
}

namespace {
int tetgen_read(const char* node_path, const char* ele_path, double natural_scale, double* rest, uint32_t max_nodes,
                uint32_t* tets, uint32_t max_tets, uint32_t* num_nodes, uint32_t* num_tets, uint32_t* num_dropped)
{
    if (!node_path || !ele_path || !num_nodes || !num_tets)
        return io_fail(FEM_E_ARG, "null path or count output");
    if (!(natural_scale >= 0) || !std::isfinite(natural_scale))
        return io_fail(FEM_E_ARG, "natural_scale must be finite and >= 0 (0: none)");
    std::vector<float> pos;
    long base_vid = 0;
    {
        File nf;
        nf.f = std::fopen(node_path, "r");
        if (!nf.f) return io_fail(FEM_E_ARG, std::string("cannot open ") + node_path);
        Tokens tk(nf.f);
        long n = 0, dim = 0, nattr = 0, nbnd = 0;
        if (!tk.next_long(n) || !tk.next_long(dim) || !tk.next_long(nattr) || !tk.next_long(nbnd))
            return io_fail(FEM_E_ARG, std::string(node_path) + ": malformed header");
        if (dim != 3) return io_fail(FEM_E_ARG, std::string(node_path) + ": dimension is not 3");
        if (n <= 0 || n > (1L << 30) || nattr < 0 || nbnd < 0 || nbnd > 1)
            return io_fail(FEM_E_ARG, std::string(node_path) + ": bad counts in the header");
        // grown as nodes are read, so a header that promises more nodes than
        // the file holds fails on the missing lines, not on the allocation
        pos.reserve(3 * (size_t)std::min(n, 1L << 20));
        for (long i = 0; i < n; i++) {
            long vid = 0;
            float p[3];
            if (!tk.next_long(vid) || !tk.next_float(p[0]) || !tk.next_float(p[1]) || !tk.next_float(p[2]))
                return io_fail(FEM_E_ARG, std::string(node_path) + ": malformed node " + std::to_string(i));
            pos.insert(pos.end(), p, p + 3);
            if (i == 0) base_vid = vid;
            float dummy;
            for (long a = 0; a < nattr + nbnd; a++)
                if (!tk.next_float(dummy))
                    return io_fail(FEM_E_ARG, std::string(node_path) + ": malformed node " + std::to_string(i));
        }
    }
    const long N = (long)(pos.size() / 3);
    std::vector<uint32_t> kept;
    uint32_t dropped = 0;
    {
        File ef;
        ef.f = std::fopen(ele_path, "r");
        if (!ef.f) return io_fail(FEM_E_ARG, std::string("cannot open ") + ele_path);
        Tokens tk(ef.f);
        long t = 0, npt = 0, nattr = 0;
        if (!tk.next_long(t) || !tk.next_long(npt) || !tk.next_long(nattr))
            return io_fail(FEM_E_ARG, std::string(ele_path) + ": malformed header");
        if (npt != 4) return io_fail(FEM_E_ARG, std::string(ele_path) + ": not 4 nodes per tet (linear tets only)");
        if (t <= 0 || t > (1L << 29) || nattr < 0)
            return io_fail(FEM_E_ARG, std::string(ele_path) + ": bad counts in the header");
        kept.reserve(4 * (size_t)std::min(t, 1L << 20));
        for (long e = 0; e < t; e++) {
            long tid = 0, v[4];
            if (!tk.next_long(tid) || !tk.next_long(v[0]) || !tk.next_long(v[1]) || !tk.next_long(v[2]) ||
                !tk.next_long(v[3]))
                return io_fail(FEM_E_ARG, std::string(ele_path) + ": malformed tet " + std::to_string(e));
            float dummy;
            for (long a = 0; a < nattr; a++)
                if (!tk.next_float(dummy))
                    return io_fail(FEM_E_ARG, std::string(ele_path) + ": malformed tet " + std::to_string(e));
            for (int k = 0; k < 4; k++) {
                v[k] -= base_vid;
                if (v[k] < 0 || v[k] >= N)
                    return io_fail(FEM_E_INDEX, std::string(ele_path) + ": tet " + std::to_string(e) +
                                                    " names a node outside the .node file");
            }
            const float* p0 = &pos[3 * v[0]];
            float c1[3], c2[3], c3[3];
            for (int a = 0; a < 3; a++) {
                c1[a] = pos[3 * v[1] + a] - p0[a];
                c2[a] = pos[3 * v[2] + a] - p0[a];
                c3[a] = pos[3 * v[3] + a] - p0[a];
            }
            if (det_columns(c1, c2, c3) <= 0.0f) {
                dropped++;
                continue;
            }
            for (int k = 0; k < 4; k++) kept.push_back((uint32_t)v[k]);
        }
    }
    if (natural_scale > 0) {
        // GAABB::SetMinMax / Merge in float, node by node
        float c[3], h[3];
        for (int a = 0; a < 3; a++) {
            c[a] = 0.5f * (pos[a] + pos[a]);
            h[a] = 0.5f * (pos[a] - pos[a]);
        }
        for (long i = 1; i < N; i++)
            for (int a = 0; a < 3; a++) {
                float lo = c[a] - h[a], hi = c[a] + h[a];
                const float p = pos[3 * i + a];
                lo = (p < lo) ? p : lo;
                hi = (p > hi) ? p : hi;
                c[a] = 0.5f * (lo + hi);
                h[a] = 0.5f * (hi - lo);
            }
        float ext = 2 * h[0];
        if (2 * h[1] > ext) ext = 2 * h[1];
        if (2 * h[2] > ext) ext = 2 * h[2];
        // one node, or every node at one point: nothing to scale to the
        // requested size (the converter would divide by zero)
        if (!(ext > 0.0f) || !std::isfinite(ext))
            return io_fail(FEM_E_ARG, "natural_scale: the nodes span no extent (" + std::to_string(ext) + ")");
        const float s = (float)natural_scale / ext;
        for (long i = 0; i < N; i++)
            for (int a = 0; a < 3; a++) {
                const float moved = pos[3 * i + a] + (-c[a]);
                pos[3 * i + a] = s * moved;
            }
    }
    *num_nodes = (uint32_t)N;
    *num_tets = (uint32_t)(kept.size() / 4);
    if (num_dropped) *num_dropped = dropped;
    if (rest || tets) {
        if (!rest || !tets) return io_fail(FEM_E_ARG, "give both output arrays, or neither to query the sizes");
        if (max_nodes < (uint32_t)N || max_tets < *num_tets)
            return io_fail(FEM_E_ARG, "output arrays too small for the mesh");
        for (size_t i = 0; i < pos.size(); i++) rest[i] = (double)pos[i];
        std::memcpy(tets, kept.data(), sizeof(uint32_t) * kept.size());
    }
    return FEM_OK;
}
}  // namespace

// shape_io.cpp -- the tetrahedral solid shape of the reference's geometry
// library (host only): EditableTetSolidShape3::EndEdition's rebuild and the
// shape-library text file (.geo) that its TetGen converter writes and its
// solids load.
//
// The solid the reference simulates is built from a TetSolidShape3: its
// vertices (float) and its tets in the shape's order
// (LeafDSH_Solid3D_FEM.cpp:158-168 adds the shape's tets to the element set
// one by one). EndEdition (Geo/shape/TetSolidShape3.cpp:558-565) changes
// both before that:
//   1. FixDegenerateVertices (:809-845): vertices no tet references are
//      removed, the others keep their order;
//   2. RebuildTopology (:619-748): each tet's neighbour across the face
//      opposite each of its vertices (the tet sharing that face's three
//      vertices; faces met in tet order, a face matched against every
//      earlier face with the same vertices), and one boundary face per
//      unmatched face, oriented outwards by the sign of
//      dot(x_opp - x_a, cross(x_b - x_a, x_c - x_a)) in float;
//   3. RebuildLayers (:752-807): vertex layers (0 on the boundary faces,
//      else one more than the lowest neighbour in a tet: the breadth-first
//      distance the reference reaches by relaxation), tet layer = the lowest
//      of its vertices', tets reordered by layer (stable) and the neighbour
//      ids renumbered.
// The .geo file: ShapeLibrary::Register_TetSolidShape3
// (Geo/shape/ShapeLibrary.cpp:332-360) written by ItemStream's text form
// (util/ItemStreamSerialization.cpp:14-182): one complex item "#1" holding
// shape_type (21, eShape_TetSolid3), version (3), the counts, and the
// baked arrays as hex byte strings -- float[3] per vertex, one byte per
// vertex (an unused field; written as 0), uint16 vids[4] + neighbour ids[4]
// per tet, uint16 vids[3] per boundary face, uint16 (first, count) per
// layer. The shape's indices are uint16 (0xFFFF = none), so a shape file
// holds at most 65534 vertices and tets.
#include "../../include/fem_tet.h"

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

namespace femgb {
void set_last_error(const char* msg);
}

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kShapeTetSolid3 = 21;  // eShape_TetSolid3 (Geo/ShapeTypes.h)
constexpr uint32_t kShapeVersion = 3;     // TetSolidShape3::cVersion
constexpr uint32_t kGeoMaxFeatures = 0xFFFEu;

int shape_fail(int code, const std::string& msg)
{
    femgb::set_last_error(msg.c_str());
    return code;
}

struct Shape {
    std::vector<float> pos;       // 3 V
    std::vector<uint32_t> vmap;   // input vertex -> shape vertex (kNone: removed)
    std::vector<uint32_t> tets;   // 4 T, shape vertex ids, layer order
    std::vector<uint32_t> ntid;   // 4 T, neighbour across the face opposite vertex i (kNone: boundary)
    std::vector<uint32_t> tperm;  // shape tet -> input tet
    std::vector<uint32_t> bf;     // 3 per boundary face
    std::vector<uint32_t> layers; // (first, count) per layer
};

struct FaceKey {
    uint32_t a, b, c;
    bool operator<(const FaceKey& o) const
    {
        if (a != o.a) return a < o.a;
        if (b != o.b) return b < o.b;
        return c < o.c;
    }
    bool operator==(const FaceKey& o) const { return a == o.a && b == o.b && c == o.c; }
};

FaceKey face_key(uint32_t x, uint32_t y, uint32_t z)
{
    if (x > y) std::swap(x, y);
    if (y > z) std::swap(y, z);
    if (x > y) std::swap(x, y);
    return FaceKey{x, y, z};
}

// The rebuild; the tets are valid (ids < N) and positions finite.
void rebuild(const float* pos, uint32_t N, const uint32_t* tets_in, uint32_t T, Shape& s)
{
    // 1. unreferenced vertices out
    std::vector<uint32_t> degree(N, 0);
    for (size_t k = 0; k < 4ull * T; k++) degree[tets_in[k]]++;
    s.vmap.assign(N, kNone);
    s.pos.clear();
    for (uint32_t v = 0; v < N; v++)
        if (degree[v] > 0) {
            s.vmap[v] = (uint32_t)(s.pos.size() / 3);
            s.pos.insert(s.pos.end(), pos + 3 * (size_t)v, pos + 3 * (size_t)v + 3);
        }
    const uint32_t V = (uint32_t)(s.pos.size() / 3);
    std::vector<uint32_t> t0(4ull * T), n0(4ull * T, kNone);
    for (size_t k = 0; k < 4ull * T; k++) t0[k] = s.vmap[tets_in[k]];

    // 2. neighbours and boundary faces. Faces with the same three vertices
    // form a group in the order they are met; each face met is matched
    // against every earlier one of its group (the later match overwriting),
    // so the last face of a group points at the one before it and every
    // other face at the last.
    s.bf.clear();
    if (V > 0 && T > 0) {
        std::vector<std::pair<FaceKey, uint32_t>> faces(4ull * T);
        for (uint32_t t = 0; t < T; t++)
            for (uint32_t n = 0; n < 4; n++) {
                const uint32_t* q = &t0[4ull * t];
                faces[4ull * t + n] = {face_key(q[(n + 1) & 3], q[(n + 2) & 3], q[(n + 3) & 3]), 4 * t + n};
            }
        std::stable_sort(faces.begin(), faces.end(),
                         [](const std::pair<FaceKey, uint32_t>& x, const std::pair<FaceKey, uint32_t>& y) {
                             return x.first < y.first;
                         });
        for (size_t i = 0; i < faces.size();) {
            size_t j = i + 1;
            while (j < faces.size() && faces[j].first == faces[i].first) j++;
            const size_t m = j - i;
            if (m >= 2) {
                const uint32_t last = faces[j - 1].second, prev = faces[j - 2].second;
                for (size_t k = i; k + 1 < j; k++) n0[faces[k].second] = last >> 2;
                n0[last] = prev >> 2;
            }
            i = j;
        }
        for (uint32_t t = 0; t < T; t++)
            for (uint32_t n = 0; n < 4; n++) {
                if (n0[4ull * t + n] != kNone) continue;
                const uint32_t* q = &t0[4ull * t];
                const uint32_t a = q[(n + 1) & 3], b = q[(n + 2) & 3], c = q[(n + 3) & 3], o = q[n];
                const float* pa = &s.pos[3ull * a];
                const float* pb = &s.pos[3ull * b];
                const float* pc = &s.pos[3ull * c];
                const float* po = &s.pos[3ull * o];
                const float e1[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
                const float e2[3] = {pc[0] - pa[0], pc[1] - pa[1], pc[2] - pa[2]};
                const float d[3] = {po[0] - pa[0], po[1] - pa[1], po[2] - pa[2]};
                const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                     e1[0] * e2[1] - e1[1] * e2[0]};
                float dot = 0.f;
                dot += d[0] * cr[0];
                dot += d[1] * cr[1];
                dot += d[2] * cr[2];
                if (dot <= 0.f) {
                    s.bf.push_back(a); s.bf.push_back(b); s.bf.push_back(c);
                } else {
                    s.bf.push_back(a); s.bf.push_back(c); s.bf.push_back(b);
                }
            }
    }

    // 3. layers: breadth-first distance from the boundary vertices over
    // "shares a tet" (the fixed point of the reference's relaxation, which
    // runs T sweeps: a shortest path of d hops passes d distinct tets)
    const uint32_t cap = T;
    std::vector<uint32_t> vl(V, cap);
    std::deque<uint32_t> queue;
    for (uint32_t v : s.bf)
        if (vl[v] != 0) {
            vl[v] = 0;
            queue.push_back(v);
        }
    if (!queue.empty()) {
        // vertex -> tets
        std::vector<uint32_t> vptr(V + 1, 0), vt(4ull * T);
        for (size_t k = 0; k < 4ull * T; k++) vptr[t0[k] + 1]++;
        for (uint32_t v = 0; v < V; v++) vptr[v + 1] += vptr[v];
        std::vector<uint32_t> fill(vptr.begin(), vptr.end() - 1);
        for (uint32_t t = 0; t < T; t++)
            for (int i = 0; i < 4; i++) vt[fill[t0[4ull * t + i]]++] = t;
        while (!queue.empty()) {
            const uint32_t v = queue.front();
            queue.pop_front();
            for (uint32_t k = vptr[v]; k < vptr[v + 1]; k++) {
                const uint32_t* q = &t0[4ull * vt[k]];
                for (int i = 0; i < 4; i++)
                    if (vl[q[i]] > vl[v] + 1) {
                        vl[q[i]] = vl[v] + 1;
                        queue.push_back(q[i]);
                    }
            }
        }
    }
    std::vector<uint32_t> tl(T, cap);
    uint32_t max_layer = 0;
    for (uint32_t t = 0; t < T; t++) {
        for (int i = 0; i < 4; i++) tl[t] = std::min(tl[t], vl[t0[4ull * t + i]]);
        max_layer = std::max(max_layer, tl[t]);
    }
    const uint32_t nl = max_layer + 1;
    std::vector<uint32_t> lcount(nl, 0);
    for (uint32_t t = 0; t < T; t++) lcount[tl[t]]++;
    s.layers.assign(2ull * nl, 0);
    std::vector<uint32_t> lnext(nl);
    uint32_t first = 0;
    for (uint32_t l = 0; l < nl; l++) {
        s.layers[2 * l] = first;
        s.layers[2 * l + 1] = lcount[l];
        lnext[l] = first;
        first += lcount[l];
    }
    std::vector<uint32_t> old2new(T);
    s.tperm.assign(T, 0);
    for (uint32_t t = 0; t < T; t++) {
        old2new[t] = lnext[tl[t]]++;
        s.tperm[old2new[t]] = t;
    }
    s.tets.assign(4ull * T, 0);
    s.ntid.assign(4ull * T, kNone);
    for (uint32_t t = 0; t < T; t++)
        for (int i = 0; i < 4; i++) {
            s.tets[4ull * old2new[t] + i] = t0[4ull * t + i];
            const uint32_t nb = n0[4ull * t + i];
            s.ntid[4ull * old2new[t] + i] = nb == kNone ? kNone : old2new[nb];
        }
}

int check_mesh(const double* rest, uint32_t N, const uint32_t* tets, uint32_t T)
{
    if ((N && !rest) || (T && !tets)) return shape_fail(FEM_E_ARG, "null mesh arrays");
    for (size_t k = 0; k < 4ull * T; k++)
        if (tets[k] >= N)
            return shape_fail(FEM_E_INDEX, "tet " + std::to_string(k / 4) + " names node " + std::to_string(tets[k]) +
                                                " >= N=" + std::to_string(N));
    return FEM_OK;
}

// ---- text form ----
void put_hex(std::string& out, const void* data, size_t bytes)
{
    static const char kHex[] = "0123456789ABCDEF";
    const unsigned char* p = static_cast<const unsigned char*>(data);
    out.reserve(out.size() + 2 * bytes + 1);
    for (size_t i = 0; i < bytes; i++) {
        out.push_back(kHex[p[i] >> 4]);
        out.push_back(kHex[p[i] & 15]);
    }
}

void put_u16(std::vector<unsigned char>& b, uint32_t v)
{
    const uint16_t w = (uint16_t)v;
    b.push_back((unsigned char)(w & 0xff));
    b.push_back((unsigned char)(w >> 8));
}

std::string geo_text(const Shape& s)
{
    const uint32_t V = (uint32_t)(s.pos.size() / 3), T = (uint32_t)(s.tets.size() / 4);
    const uint32_t NBF = (uint32_t)(s.bf.size() / 3), NL = (uint32_t)(s.layers.size() / 2);
    const std::string ind = "    ";
    std::string out = "#1\n{\n";
    char line[96];
    const std::pair<const char*, uint32_t> scalars[] = {
        {"shape_type", kShapeTetSolid3}, {"version", kShapeVersion}, {"num_v", V}, {"num_t", T},
        {"num_bf", NBF}, {"num_l", NL}};
    for (const auto& sc : scalars) {
        std::snprintf(line, sizeof(line), "%s%s %du\n", ind.c_str(), sc.first, (int)sc.second);
        out += line;
    }
    // little-endian images of the baked arrays
    std::vector<unsigned char> bytes;
    out += ind + "vec_points ^";
    for (size_t k = 0; k < s.pos.size(); k++) {
        uint32_t w;
        std::memcpy(&w, &s.pos[k], 4);
        for (int i = 0; i < 4; i++) bytes.push_back((unsigned char)(w >> (8 * i)));
    }
    put_hex(out, bytes.data(), bytes.size());
    out += "\n" + ind + "vec_v ^";
    bytes.assign(V, 0);
    put_hex(out, bytes.data(), bytes.size());
    out += "\n" + ind + "vec_t ^";
    bytes.clear();
    for (uint32_t t = 0; t < T; t++) {
        for (int i = 0; i < 4; i++) put_u16(bytes, s.tets[4ull * t + i]);
        for (int i = 0; i < 4; i++) put_u16(bytes, s.ntid[4ull * t + i] == kNone ? 0xFFFFu : s.ntid[4ull * t + i]);
    }
    put_hex(out, bytes.data(), bytes.size());
    out += "\n" + ind + "vec_bf ^";
    bytes.clear();
    for (uint32_t v : s.bf) put_u16(bytes, v);
    put_hex(out, bytes.data(), bytes.size());
    out += "\n" + ind + "vec_l ^";
    bytes.clear();
    for (uint32_t v : s.layers) put_u16(bytes, v);
    put_hex(out, bytes.data(), bytes.size());
    out += "\n}\n";
    return out;
}

// ---- reading: the subset of ItemStream's text grammar a shape file uses --
struct GeoItem {
    std::string name;
    char kind = 0;  // 'u' uint, 'h' hex bytes, 'c' complex
    uint64_t value = 0;
    std::vector<unsigned char> bytes;
    std::vector<GeoItem> sub;
};

class GeoParser {
public:
    explicit GeoParser(const std::string& t) : t_(t) {}
    bool items(std::vector<GeoItem>& out, bool nested)
    {
        for (;;) {
            skip_ws();
            if (p_ >= t_.size()) return !nested;
            if (t_[p_] == '}') {
                if (!nested) return false;
                p_++;
                return true;
            }
            GeoItem it;
            if (!item(it)) return false;
            out.push_back(std::move(it));
        }
    }
    std::string error;

private:
    const std::string& t_;
    size_t p_ = 0;
    void skip_ws()
    {
        while (p_ < t_.size() && std::isspace((unsigned char)t_[p_])) p_++;
    }
    bool fail(const char* what)
    {
        error = std::string(what) + " at byte " + std::to_string(p_);
        return false;
    }
    bool item(GeoItem& it)
    {
        size_t b = p_;
        while (p_ < t_.size() && !std::isspace((unsigned char)t_[p_])) p_++;
        it.name = t_.substr(b, p_ - b);
        if (it.name.empty()) return fail("item name expected");
        skip_ws();
        if (p_ >= t_.size()) return fail("item value expected");
        const char c = t_[p_];
        if (c == '{') {
            p_++;
            it.kind = 'c';
            return items(it.sub, true);
        }
        if (c == '^') {
            p_++;
            it.kind = 'h';
            auto hexval = [](char h) -> int {
                if (h >= '0' && h <= '9') return h - '0';
                if (h >= 'A' && h <= 'F') return h - 'A' + 10;
                if (h >= 'a' && h <= 'f') return h - 'a' + 10;
                return -1;
            };
            for (;;) {
                if (p_ >= t_.size() || std::isspace((unsigned char)t_[p_])) break;
                if (p_ + 1 >= t_.size()) return fail("odd hex string");
                const int hi = hexval(t_[p_]), lo = hexval(t_[p_ + 1]);
                if (hi < 0 || lo < 0) return fail("bad hex digit");
                it.bytes.push_back((unsigned char)(hi * 16 + lo));
                p_ += 2;
            }
            return true;
        }
        // a scalar: digits with a type suffix; only unsigned ("u") is used
        b = p_;
        while (p_ < t_.size() && !std::isspace((unsigned char)t_[p_])) p_++;
        const std::string tok = t_.substr(b, p_ - b);
        if (tok.size() >= 2 && tok.back() == 'u') {
            char* end = nullptr;
            const long long v = std::strtoll(tok.c_str(), &end, 10);
            if (end != tok.c_str() + tok.size() - 1) return fail("bad unsigned value");
            it.kind = 'u';
            it.value = (uint64_t)(uint32_t)v;
            return true;
        }
        it.kind = '?';  // other value types: kept as unknown, not needed here
        return true;
    }
};

const GeoItem* find(const std::vector<GeoItem>& items, const char* name)
{
    for (const auto& it : items)
        if (it.name == name) return &it;
    return nullptr;
}

int read_file(const char* path, std::string& text)
{
    if (!path) return shape_fail(FEM_E_ARG, "null path");
    FILE* f = std::fopen(path, "rb");
    if (!f) return shape_fail(FEM_E_ARG, std::string("cannot open ") + path);
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, n);
    std::fclose(f);
    return FEM_OK;
}

// The tet-solid shape of a shape file: its vertices, tets and neighbours.
int load_geo(const char* path, std::vector<float>& pos, std::vector<uint32_t>& tets, std::vector<uint32_t>& ntid)
{
    std::string text;
    if (int e = read_file(path, text)) return e;
    GeoParser parser(text);
    std::vector<GeoItem> top;
    if (!parser.items(top, false)) return shape_fail(FEM_E_ARG, std::string("malformed shape file: ") + parser.error);
    for (const auto& c : top) {
        if (c.kind != 'c') continue;
        const GeoItem* st = find(c.sub, "shape_type");
        if (!st || st->kind != 'u' || st->value != kShapeTetSolid3) continue;
        const GeoItem* ver = find(c.sub, "version");
        if (!ver || ver->kind != 'u' || ver->value != kShapeVersion)
            return shape_fail(FEM_E_ARG, "tet-solid shape of another version than 3");
        const GeoItem *nv = find(c.sub, "num_v"), *nt = find(c.sub, "num_t");
        const GeoItem *vp = find(c.sub, "vec_points"), *vt = find(c.sub, "vec_t");
        if (!nv || !nt || !vp || !vt || nv->kind != 'u' || nt->kind != 'u' || vp->kind != 'h' || vt->kind != 'h')
            return shape_fail(FEM_E_ARG, "tet-solid shape without its counts or arrays");
        const uint64_t V = nv->value, T = nt->value;
        if (vp->bytes.size() != 12 * V || vt->bytes.size() != 16 * T)
            return shape_fail(FEM_E_ARG, "tet-solid shape arrays do not match its counts");
        pos.resize(3 * V);
        for (size_t k = 0; k < 3 * V; k++) {
            uint32_t w = 0;
            for (int i = 0; i < 4; i++) w |= (uint32_t)vp->bytes[4 * k + i] << (8 * i);
            std::memcpy(&pos[k], &w, 4);
        }
        tets.resize(4 * T);
        ntid.resize(4 * T);
        for (size_t t = 0; t < T; t++)
            for (int i = 0; i < 4; i++) {
                const unsigned char* q = &vt->bytes[16 * t];
                const uint32_t v = q[2 * i] | ((uint32_t)q[2 * i + 1] << 8);
                const uint32_t nb = q[8 + 2 * i] | ((uint32_t)q[8 + 2 * i + 1] << 8);
                if (v >= V) return shape_fail(FEM_E_INDEX, "tet " + std::to_string(t) + " names vertex " +
                                                               std::to_string(v) + " >= num_v");
                tets[4 * t + i] = v;
                ntid[4 * t + i] = nb == 0xFFFFu ? kNone : nb;
            }
        return FEM_OK;
    }
    return shape_fail(FEM_E_ARG, "no tet-solid shape in the file");
}

int write_text(const char* path, const std::string& text)
{
    if (!path) return shape_fail(FEM_E_ARG, "null path");
    FILE* f = std::fopen(path, "wb");
    if (!f) return shape_fail(FEM_E_ARG, std::string("cannot write ") + path);
    const bool ok = std::fwrite(text.data(), 1, text.size(), f) == text.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) return shape_fail(FEM_E_ARG, std::string("write failed: ") + path);
    return FEM_OK;
}

}  // namespace

extern "C" {

int fem_tetshape_rebuild(const double* rest, uint32_t N, const uint32_t* tets, uint32_t T, double* out_rest,
                         uint32_t* out_num_nodes, uint32_t* out_tets, uint32_t* out_neighbors, uint32_t* out_tet_of,
                         uint32_t* out_node_of, uint32_t* out_bfaces, uint32_t max_bfaces, uint32_t* out_num_bfaces,
                         uint32_t* out_layers, uint32_t max_layers, uint32_t* out_num_layers)
{
    if (int e = check_mesh(rest, N, tets, T)) return e;
    std::vector<float> pf(3ull * N);
    for (size_t k = 0; k < 3ull * N; k++) pf[k] = (float)rest[k];
    Shape s;
    rebuild(pf.data(), N, tets, T, s);
    const uint32_t V = (uint32_t)(s.pos.size() / 3), NBF = (uint32_t)(s.bf.size() / 3);
    const uint32_t NL = (uint32_t)(s.layers.size() / 2);
    if (out_num_nodes) *out_num_nodes = V;
    if (out_num_bfaces) *out_num_bfaces = NBF;
    if (out_num_layers) *out_num_layers = NL;
    if (out_bfaces && max_bfaces < NBF) return shape_fail(FEM_E_ARG, "boundary-face array too short");
    if (out_layers && max_layers < NL) return shape_fail(FEM_E_ARG, "layer array too short");
    if (out_rest)
        for (uint32_t v = 0; v < N; v++)
            if (s.vmap[v] != kNone)
                for (int i = 0; i < 3; i++) out_rest[3ull * s.vmap[v] + i] = rest[3ull * v + i];
    if (out_tets) std::copy(s.tets.begin(), s.tets.end(), out_tets);
    if (out_neighbors) std::copy(s.ntid.begin(), s.ntid.end(), out_neighbors);
    if (out_tet_of) std::copy(s.tperm.begin(), s.tperm.end(), out_tet_of);
    if (out_node_of)
        for (uint32_t v = 0; v < N; v++)
            if (s.vmap[v] != kNone) out_node_of[s.vmap[v]] = v;
    if (out_bfaces) std::copy(s.bf.begin(), s.bf.end(), out_bfaces);
    if (out_layers) std::copy(s.layers.begin(), s.layers.end(), out_layers);
    return FEM_OK;
}

int fem_geo_write(const char* path, const double* rest, uint32_t N, const uint32_t* tets, uint32_t T)
{
    if (int e = check_mesh(rest, N, tets, T)) return e;
    if (N > kGeoMaxFeatures || T > kGeoMaxFeatures)
        return shape_fail(FEM_E_ARG, "a shape file holds at most 65534 vertices and tets (uint16 ids)");
    std::vector<float> pf(3ull * N);
    for (size_t k = 0; k < 3ull * N; k++) pf[k] = (float)rest[k];
    Shape s;
    rebuild(pf.data(), N, tets, T, s);
    return write_text(path, geo_text(s));
}

int fem_geo_read(const char* path, double* rest, uint32_t max_nodes, uint32_t* tets, uint32_t max_tets,
                 uint32_t* neighbors, uint32_t* num_nodes, uint32_t* num_tets)
{
    std::vector<float> pos;
    std::vector<uint32_t> t, nb;
    if (int e = load_geo(path, pos, t, nb)) return e;
    const uint32_t V = (uint32_t)(pos.size() / 3), T = (uint32_t)(t.size() / 4);
    if (num_nodes) *num_nodes = V;
    if (num_tets) *num_tets = T;
    if ((rest && max_nodes < V) || ((tets || neighbors) && max_tets < T))
        return shape_fail(FEM_E_ARG, "output arrays too short");
    if (rest)
        for (size_t k = 0; k < pos.size(); k++) rest[k] = (double)pos[k];
    if (tets) std::copy(t.begin(), t.end(), tets);
    if (neighbors) std::copy(nb.begin(), nb.end(), neighbors);
    return FEM_OK;
}

int fem_tetgen_to_geo(const char* node_path, const char* ele_path, double natural_scale, const char* geo_path)
{
    uint32_t N = 0, T = 0;
    if (int e = fem_tetgen_read(node_path, ele_path, natural_scale, nullptr, 0, nullptr, 0, &N, &T, nullptr)) return e;
    std::vector<double> rest(3ull * N);
    std::vector<uint32_t> tets(4ull * T);
    if (int e = fem_tetgen_read(node_path, ele_path, natural_scale, rest.data(), N, tets.data(), T, &N, &T, nullptr))
        return e;
    return fem_geo_write(geo_path, rest.data(), N, tets.data(), T);
}

}  // extern "C"

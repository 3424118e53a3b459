// Test infrastructure: drives the reference's own tet-solid shape and shape
// library code (src/Geo/shape/TetSolidShape3.cpp, ShapeLibrary.cpp,
// src/util/ItemStream*.cpp, compiled as written by the Makefile's "ref"
// target) the way its TetGen converter does (examples/tetgen2geo/main.cpp):
// every vertex and tet added (AddTetrahedron drops tets with det <= 0), the
// optional -nsac transform (center the AABB of the vertices, then scale its
// largest extent to natural_scale), EndEdition, and the shape library saved
// as text. The checker for fem_tetshape_rebuild / fem_geo_write; nothing in
// the library links it.
#include <Geo/bv/GAABB.h>
#include <Geo/bv/stats.h>
#include <Geo/np/Overlap.h>
#include <Geo/shape/ShapeLibrary.h>
#include <Geo/shape/TetSolidShape3.h>
#include <Geo/shape/TriSurfaceShape3.h>

// Collision-query symbols TetSolidShape3.cpp references from code the
// harness never runs (bounding-volume statistics, the point-in-tet overlap
// of its detailed collision representation, surface barycenters); defined
// here so the harness links without the rest of the geometry library.
namespace geo {
namespace bv {
Stats* g_pStats = 0;
}
namespace np {
Context* g_pDefaultContext = 0;
bool Overlap_Point3_Tetrahedron3(const Vec3&, const Vec3&, const Vec3&, const Vec3&, const Vec3&, OverlapCache3*,
                                 const Context*)
{
    return false;
}
}  // namespace np
Vec3 TriSurfaceShape3::T_Barycenter(uint32, const sdof_type*) const { return Vec3(0, 0, 0); }
}  // namespace geo

extern "C" int geo_ref_convert(const float* pos, unsigned N, const unsigned* tets, unsigned T, float natural_scale,
                               const char* out_path)
{
    geo::EditableTetSolidShape3 shape;
    shape.BeginEdition();
    geo::bv::AABB3 box;
    for (unsigned i = 0; i < N; i++) {
        const geo::Vec3 p(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        shape.AddVertex(p);
        if (i == 0)
            box.SetMinMax(p, p);
        else
            box.Merge(p);
    }
    for (unsigned t = 0; t < T; t++) shape.AddTetrahedron(tets[4 * t], tets[4 * t + 1], tets[4 * t + 2], tets[4 * t + 3]);
    if (natural_scale > 0.f) {
        const float s = natural_scale / mal::Max(2 * box.GetHalfSizes());
        shape.Transform(geo::Transform3(-box.GetPos(), geo::Mat3x3::Identity()));
        shape.Transform(geo::Transform3(geo::Vec3::Zero(), mal::GMatNxN_From_Diagonal(geo::Vec3(s, s, s))));
    }
    shape.EndEdition();
    geo::ShapeLibrary lib;
    lib.Reserve(1 << 24);
    lib.Register(shape);
    return lib.Save(out_path, false) ? 0 : 1;
}

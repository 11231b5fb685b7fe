// Test infrastructure: drives libmat's own Houdini geometry writer
// (IO::Geometry / IO::GeometryWriter, src/IO/IO_CUDA/io_utils.cpp:106-231)
// the way save_convex_cells_houdini (src/IO/IO_CUDA/io_cuda.cxx:156-187)
// calls it: point attribute "P", the polygons, primitive attribute
// "PrimAttr" = the polygon's site.  Compiled with the reference's sources by
// oracle/build.py into oracle/_ref/librefbgeo.so; the tests compare the
// oracle's writer and the device's file with the file it writes.
#include <stdexcept>
#include <string>
#include <vector>

#include "io_utils.hpp"

extern "C" int ref_write_bgeo(const char* folder, const char* name, const float* points,
                              long long n_points, const long long* poly_offsets,
                              const unsigned* indices, long long n_polys, const int* poly_site) {
  std::vector<float3> p((size_t)n_points);
  for (long long i = 0; i < n_points; ++i) p[i] = float3{points[3 * i], points[3 * i + 1], points[3 * i + 2]};
  std::vector<std::vector<unsigned>> faces((size_t)n_polys);
  for (long long i = 0; i < n_polys; ++i)
    faces[i].assign(indices + poly_offsets[i], indices + poly_offsets[i + 1]);
  std::vector<int> sites(poly_site, poly_site + n_polys);
  try {
    IO::Geometry geometry;
    IO::GeometryWriter writer(folder);
    geometry.AddParticleAttribute("P", p);
    geometry.AddPolygon(faces);
    geometry.AddPrimitiveAttribute("PrimAttr", sites);
    writer.OutputGeometry(name, geometry);
  } catch (const std::exception&) {
    return 1;
  }
  return 0;
}

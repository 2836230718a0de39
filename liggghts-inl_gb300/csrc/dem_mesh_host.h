// Host-side mesh preparation (dem_mesh_host.cu).
#pragma once
#include <cstdint>
#include <vector>

namespace gb300 {

struct MeshHost {
  int ntri = 0;
  std::vector<double> tri;     // [t*kTriStride] geometry, layout of MeshDev::tri
  std::vector<int> meta;       // obtuse index + edge/corner activity bits
  std::vector<uint8_t> edge_active, corner_active;  // [t*3]
  std::vector<int> cn_start, cn_list;               // coplanar node-neighbours
  std::vector<double> bbox;    // [t*6]: lower then upper corner of each triangle (initial mesh)
};

// Geometry, topology (unless edge/corner activity are given) and coplanar
// neighbour lists of a triangle mesh, nodes[ntri][3][3] in element order.
int mesh_prepare(int ntri, const double *nodes, const uint8_t *edge_active,
                 const uint8_t *corner_active, MeshHost &out);

}  // namespace gb300

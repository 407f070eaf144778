// reader_stub.h -- the mesh the driver hands to fe::Mesh through the stub
// readMshFile (TEST INFRASTRUCTURE ONLY, oracle/refshim).
#pragma once

#include <cstddef>
#include <vector>

#include "util/point.h"

struct InjectedMesh {
  std::vector<util::Point3> nodes;
  size_t element_type = 0;  // VTK cell type
  size_t vertices = 0;      // nodes per element
  std::vector<size_t> enc;  // element-node connectivity, flat
};

extern InjectedMesh g_injected_mesh;

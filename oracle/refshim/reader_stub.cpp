// reader_stub.cpp -- the mesh-file readers fe/mesh.cpp links against.
//
// TEST INFRASTRUCTURE ONLY (oracle/refshim).  The reference's rw/reader.cpp
// needs VTK and Gmsh; the refshim hands nodes and volumes to
// fe::Mesh::setMeshData instead, so these entry points throw if they are
// reached, except readMshFile, which hands over a mesh the driver put in
// g_injected_mesh (nodes, element type, connectivity) so that the reference's
// fe::Mesh::createData and computeVol run on it.
#include <stdexcept>
#include <string>
#include <vector>

#include "rw/reader.h"
#include "reader_stub.h"

namespace {
[[noreturn]] void unavailable(const char *what) {
  throw std::runtime_error(std::string("mesh reader not available in the refshim: ") + what);
}
}  // namespace

void rw::reader::readCsvFile(const std::string &, size_t, std::vector<util::Point3> *,
                             std::vector<double> *) {
  unavailable("csv");
}
void rw::reader::readVtuFileNodes(const std::string &, size_t, std::vector<util::Point3> *,
                                  bool) {
  unavailable("vtu nodes");
}
void rw::reader::readVtuFileCells(const std::string &, size_t, size_t &, size_t &,
                                  std::vector<size_t> *, std::vector<std::vector<size_t>> *) {
  unavailable("vtu cells");
}
bool rw::reader::readVtuFilePointData(const std::string &, const std::string &,
                                      std::vector<uint8_t> *) {
  unavailable("vtu point data");
}
bool rw::reader::readVtuFilePointData(const std::string &, const std::string &,
                                      std::vector<size_t> *) {
  unavailable("vtu point data");
}
bool rw::reader::readVtuFilePointData(const std::string &, const std::string &,
                                      std::vector<double> *) {
  unavailable("vtu point data");
}
bool rw::reader::readVtuFilePointData(const std::string &, const std::string &,
                                      std::vector<util::Point3> *) {
  unavailable("vtu point data");
}
InjectedMesh g_injected_mesh;

// The node-element lists as MshReader::readMesh forms them
// (mshReader.cpp:95-113): element ids in connectivity order.
void rw::reader::readMshFile(const std::string &, size_t, std::vector<util::Point3> *nodes,
                             size_t &element_type, size_t &num_elem, std::vector<size_t> *enc,
                             std::vector<std::vector<size_t>> *nec, std::vector<double> *volumes,
                             bool) {
  const InjectedMesh &m = g_injected_mesh;
  if (m.nodes.empty()) unavailable("msh");
  *nodes = m.nodes;
  element_type = m.element_type;
  *enc = m.enc;
  volumes->clear();
  nec->assign(m.nodes.size(), {});
  const size_t nv = m.vertices;
  for (size_t j = 0; j < m.enc.size(); j++) (*nec)[m.enc[j]].push_back(j / nv);
  num_elem = m.enc.size() / nv;
}

// reader_stub.cpp -- the mesh-file readers fe/mesh.cpp links against.
//
// TEST INFRASTRUCTURE ONLY (oracle/refshim).  The reference's rw/reader.cpp
// needs VTK and Gmsh; the refshim hands nodes and volumes to
// fe::Mesh::setMeshData instead, so these entry points are never reached and
// throw if they are.
#include <stdexcept>
#include <string>
#include <vector>

#include "rw/reader.h"

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
void rw::reader::readMshFile(const std::string &, size_t, std::vector<util::Point3> *, size_t &,
                             size_t &, std::vector<size_t> *,
                             std::vector<std::vector<size_t>> *, std::vector<double> *, bool) {
  unavailable("msh");
}

/*
 * ORACLE harness shim (project code).  Stands in for LAMMPS' Error class so
 * that the reference's sources compile outside LAMMPS.  Unlike the
 * reference's LAMMPS_STUB/error.h it never exits the process: it throws, and
 * the C wrapper in ref_capi.cpp turns that into an error return.
 */
#ifndef GFMD_REF_SHIM_ERROR_H
#define GFMD_REF_SHIM_ERROR_H
#define LMP_STUB_ERROR_H 1
#define LMP_ERROR_H 1

#include <stdexcept>
#include <string>

#define FLERR __FILE__, __LINE__

namespace LAMMPS_NS {

class Error {
 public:
  void all(const char *file, int line, const char *msg) { raise(file, line, msg); }
  void one(const char *file, int line, const char *msg) { raise(file, line, msg); }
  void warning(const char *, int, const char *, int = 1) {}
 private:
  static void raise(const char *file, int line, const char *msg) {
    throw std::runtime_error(std::string(file) + ":" + std::to_string(line) + ": " + msg);
  }
};

}  // namespace LAMMPS_NS

#endif

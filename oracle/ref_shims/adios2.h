/* Stand-in for the part of ADIOS2 2.6's C++ API that VoxelsCA::WriteToHDF1
 * (VoxelsCA.C:1818-1854) uses. Test infrastructure: instead of an HDF5 file it
 * writes each Put() array as raw little-endian bytes to
 * "$CAFE_REF_DUMP_DIR/<file>.<variable>.bin" when CAFE_REF_DUMP_DIR is set, and
 * writes nothing otherwise. */
#ifndef CAFE_REF_SHIM_ADIOS2_H
#define CAFE_REF_SHIM_ADIOS2_H
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include "mpi.h"

namespace adios2 {
using Dims = std::vector<size_t>;
enum class Mode { Write, Read };

template <class T> class Variable {
 public:
  std::string name;
  Dims count;
};

class Engine {
 public:
  std::string file;
  template <class T> void Put(const Variable<T> &v, const T *data) {
    const char *dir = std::getenv("CAFE_REF_DUMP_DIR");
    if (!dir || !data) return;
    size_t n = 1;
    for (size_t c : v.count) n *= c;
    std::string base = file;
    size_t slash = base.find_last_of('/');
    if (slash != std::string::npos) base = base.substr(slash + 1);
    std::string path = std::string(dir) + "/" + base + "." + v.name + ".bin";
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return;
    std::fwrite(data, sizeof(T), n, fp);
    std::fclose(fp);
  }
  void Close() {}
};

class IO {
 public:
  void SetEngine(const std::string &) {}
  template <class T>
  Variable<T> DefineVariable(const std::string &name, const Dims &, const Dims &,
                             const Dims &count) {
    Variable<T> v;
    v.name = name;
    v.count = count;
    return v;
  }
  Engine Open(const std::string &file, Mode) {
    Engine e;
    e.file = file;
    return e;
  }
};

class ADIOS {
 public:
  explicit ADIOS(MPI_Comm) {}
  IO DeclareIO(const std::string &) { return IO(); }
};
}  // namespace adios2
#endif

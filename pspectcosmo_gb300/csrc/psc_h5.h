// psc_h5.h — a minimal HDF5 file writer for the reference's snapshot files.
//
// The reference writes data_<step>_snapshot.h5 through the HDF5 C++ API
// (output.cpp:1541-1648): one contiguous H5T_IEEE_F64LE dataset of rank 3 (N x N x N)
// per field, "/ScalarField_<fld>", and with SNAPSHOTS_ENERGY the four lattice energy
// densities "/PotentialEnergy", "/KineticEnergy", "/GradientEnergy", "/TotalEnergy".
// libhdf5 is not a dependency of this library, so the file is written here in the
// HDF5 file format's original layout, which every HDF5 release reads:
//   superblock version 0 (8-byte offsets and lengths), root group = object header
//   (version 1) with a symbol-table message -> version-1 B-tree of group nodes -> symbol
//   table nodes (8 entries each, sorted by name) + a local heap with the names;
//   per dataset a version-1 object header with the dataspace (version 1), datatype
//   (IEEE float, 8 bytes, little endian), fill value (version 1, default) and layout
//   (version 3, contiguous) messages; raw data contiguous after the headers.
// Datasets are declared when the file is opened and then written one at a time, so a
// caller can stream N^3 arrays without holding them all in memory.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace psc {
namespace h5 {

class Writer {
  public:
    ~Writer();
    // Creates (truncates) `path` with datasets `names` (a leading '/' is dropped),
    // each of shape `dims` (row-major, last dimension fastest), and writes all
    // metadata. Returns 0 or -1 (see error()).
    int open(const std::string &path, const std::vector<std::string> &names, const std::vector<uint64_t> &dims);
    // The same with a shape per dataset.
    int open(const std::string &path, const std::vector<std::string> &names,
             const std::vector<std::vector<uint64_t>> &shapes);
    // Writes the whole of dataset i (in the order given to open) from `data`.
    int write(int i, const double *data);
    int close();
    const std::string &error() const { return err_; }

  private:
    int fail(const std::string &msg);
    std::FILE *fp_ = nullptr;
    std::vector<uint64_t> data_addr_, data_bytes_;
    std::string err_;
};

// Reads the files Writer writes (superblock 0, symbol-table root group, version-1
// object headers, contiguous IEEE F64LE datasets); anything else is refused.
class Reader {
  public:
    ~Reader();
    int open(const std::string &path);
    // shape of dataset `name` (a leading '/' is dropped); -1 if absent
    int shape(const std::string &name, std::vector<uint64_t> *dims);
    // reads the whole dataset (count = product of its dims) into out
    int read(const std::string &name, double *out, size_t count);
    const std::string &error() const { return err_; }

  private:
    struct Dset {
        std::vector<uint64_t> dims;
        uint64_t addr = 0, bytes = 0;
    };
    int fail(const std::string &msg);
    int get(uint64_t addr, void *dst, size_t n);
    int dataset(const std::string &name, Dset *d);
    std::FILE *fp_ = nullptr;
    uint64_t eof_ = 0;
    std::vector<std::pair<std::string, uint64_t>> links_;   // name -> object header address
    std::string err_;
};

}  // namespace h5
}  // namespace psc

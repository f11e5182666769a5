/*
 * Minimal HDF5 C++ API shim for building the reference's own sources as the CPU
 * oracle (test infrastructure only). libhdf5 is not installed here. Only the
 * names output.cpp's snapshots() uses are provided (H5std_string, hsize_t,
 * H5F_ACC_TRUNC, H5::H5File, H5::DataSet, H5::DataSpace,
 * H5::PredType::NATIVE_DOUBLE). A dataset write stores the raw little-endian
 * doubles in "<file>.<dataset>.bin" so snapshot contents can still be compared;
 * the product's own HDF5 writer lives in the package, not here.
 */
#ifndef PSC_SHIM_H5CPP_H
#define PSC_SHIM_H5CPP_H

#include <cstdio>
#include <string>
#include <vector>

typedef std::string H5std_string;
typedef unsigned long long hsize_t;
#define H5F_ACC_TRUNC 2u

namespace H5 {

struct PredType {
    int id;
    static const PredType NATIVE_DOUBLE;
};
inline const PredType PredType::NATIVE_DOUBLE = {1};

class DataSpace {
  public:
    DataSpace() {}
    DataSpace(int rank, const hsize_t *dims) : dims_(dims, dims + rank) {}
    size_t count() const {
        size_t n = 1;
        for (hsize_t d : dims_) n *= (size_t)d;
        return dims_.empty() ? 0 : n;
    }
  private:
    std::vector<hsize_t> dims_;
};

class DataSet {
  public:
    DataSet() {}
    DataSet(const std::string &path, const DataSpace &sp) : path_(path), space_(sp) {}
    void write(const void *buf, const PredType &) const {
        std::FILE *fp = std::fopen(path_.c_str(), "wb");
        if (!fp) return;
        std::fwrite(buf, sizeof(double), space_.count(), fp);
        std::fclose(fp);
    }
    void close() {}
  private:
    std::string path_;
    DataSpace space_;
};

class H5File {
  public:
    H5File(const std::string &name, unsigned) : name_(name) {}
    DataSet createDataSet(const std::string &ds, const PredType &, const DataSpace &sp) const {
        std::string clean = ds;
        for (char &c : clean) if (c == '/') c = '_';
        return DataSet(name_ + "." + clean + ".bin", sp);
    }
    void close() {}
  private:
    std::string name_;
};

} // namespace H5
#endif

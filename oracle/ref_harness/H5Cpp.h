// Stand-in for the HDF5 C++ header (test infrastructure).
//
// The reference's beam/kernel headers name H5 types in declarations of their
// file-I/O members, and the kernel source (DoseCalcIO/kernel.cpp) writes its
// cumulative kernel through them.  This header keeps the names and routes
// every dataset and attribute write into an in-memory store
// (H5::mem_datasets / H5::mem_attrs, keyed by name), so that the reference
// harness can read back exactly the arrays the reference would have stored
// in cumulative_kernel.h5.  No file is written.
#pragma once
#include <cstring>
#include <map>
#include <string>
#include <vector>

typedef unsigned long long hsize_t;
typedef std::string H5std_string;
enum { H5F_ACC_RDONLY = 0, H5F_ACC_TRUNC = 2 };
enum H5S_seloper_t { H5S_SELECT_SET = 0 };

namespace H5 {

struct MemArray {
    std::vector<hsize_t> dims;
    std::vector<unsigned char> bytes;
};
inline std::map<std::string, MemArray> mem_datasets;
inline std::map<std::string, MemArray> mem_attrs;
inline std::map<std::string, std::string> mem_str_attrs;

class CompType {};

class DataType {
  public:
    size_t size = 4;
    bool is_string = false;
    DataType() = default;
    explicit DataType(size_t s, bool str = false) : size(s), is_string(str) {}
};

class PredType : public DataType {
  public:
    explicit PredType(size_t s) : DataType(s) {}
    static const PredType NATIVE_INT, NATIVE_FLOAT, STD_U16LE, IEEE_F32LE, C_S1;
};
inline const PredType PredType::NATIVE_INT{4};
inline const PredType PredType::NATIVE_FLOAT{4};
inline const PredType PredType::STD_U16LE{2};
inline const PredType PredType::IEEE_F32LE{4};
inline const PredType PredType::C_S1{1};

class StrType : public DataType {
  public:
    StrType(const PredType&, size_t n) : DataType(n, true) {}
};

class DataSpace {
  public:
    std::vector<hsize_t> dims, off, cnt;
    DataSpace() = default;
    DataSpace(int rank, const hsize_t* d) : dims(d, d + rank), off(rank, 0), cnt(d, d + rank) {}
    void selectHyperslab(H5S_seloper_t, const hsize_t* count, const hsize_t* offset) {
        for (size_t a = 0; a < dims.size(); a++) { cnt[a] = count[a]; off[a] = offset[a]; }
    }
    int getSimpleExtentDims(hsize_t* d) const {
        for (size_t a = 0; a < dims.size(); a++) d[a] = dims[a];
        return (int)dims.size();
    }
    size_t npoints() const {
        size_t n = 1;
        for (hsize_t c : cnt) n *= c;
        return n;
    }
};

class Attribute {
  public:
    std::string name;
    DataSpace space;
    DataType type;
    DataType getDataType() const { return type; }
    void write(const DataType& t, const std::string& s) { (void)t; mem_str_attrs[name] = s; }
    // values are stored as 4-byte host words (int or float), one per element
    void write(const DataType&, const void* buf) {
        MemArray& m = mem_attrs[name];
        m.dims = space.dims;
        size_t n = space.dims.empty() ? 1 : space.npoints();
        m.bytes.assign((const unsigned char*)buf, (const unsigned char*)buf + 4 * n);
    }
    void read(const DataType&, std::string& s) const { s = mem_str_attrs[name]; }
    void read(const DataType&, void* buf) const {
        const MemArray& m = mem_attrs[name];
        std::memcpy(buf, m.bytes.data(), m.bytes.size());
    }
};

class DataSet {
  public:
    std::string name;
    DataSpace space;
    DataSpace getSpace() const { return space; }
    // row-major hyperslab copy (rank <= 3) between the store and a buffer
    void copy(const void* src, void* dst, const DataSpace& file, bool to_store) const {
        const size_t r = file.dims.size();
        hsize_t d[3] = {1, 1, 1}, o[3] = {0, 0, 0}, c[3] = {1, 1, 1};
        for (size_t a = 0; a < r; a++) {
            d[3 - r + a] = file.dims[a];
            o[3 - r + a] = file.off[a];
            c[3 - r + a] = file.cnt[a];
        }
        size_t k = 0;
        for (hsize_t i = 0; i < c[0]; i++)
            for (hsize_t j = 0; j < c[1]; j++)
                for (hsize_t l = 0; l < c[2]; l++, k++) {
                    size_t f = ((o[0] + i) * d[1] + (o[1] + j)) * d[2] + (o[2] + l);
                    if (to_store) std::memcpy((unsigned char*)dst + 4 * f, (const unsigned char*)src + 4 * k, 4);
                    else std::memcpy((unsigned char*)dst + 4 * k, (const unsigned char*)src + 4 * f, 4);
                }
    }
    void write(const void* buf, const DataType&, const DataSpace&, const DataSpace& file) const {
        MemArray& m = mem_datasets[name];
        size_t total = 1;
        for (hsize_t v : file.dims) total *= v;
        if (m.bytes.size() != 4 * total) m.bytes.assign(4 * total, 0);
        m.dims = file.dims;
        copy(buf, m.bytes.data(), file, true);
    }
    void write(const void* buf, const DataType& t, const DataSpace& file) const { write(buf, t, file, file); }
    void read(void* buf, const DataType&, const DataSpace&, const DataSpace& file) const {
        copy(mem_datasets[name].bytes.data(), buf, file, false);
    }
};

class Group {
  public:
    Attribute openAttribute(const std::string& n) const {
        Attribute a;
        a.name = n;
        return a;
    }
    Attribute createAttribute(const std::string& n, const DataType& t, const DataSpace& s) const {
        Attribute a;
        a.name = n;
        a.type = t;
        a.space = s;
        return a;
    }
    DataSet openDataSet(const std::string& n) const {
        DataSet d;
        d.name = n;
        const MemArray& m = mem_datasets[n];
        d.space = DataSpace((int)m.dims.size(), m.dims.data());
        return d;
    }
    DataSet createDataSet(const std::string& n, const DataType&, const DataSpace& s) const {
        DataSet d;
        d.name = n;
        d.space = s;
        return d;
    }
};

class H5File {
  public:
    H5File(const std::string&, unsigned) {}
    Group openGroup(const std::string&) const { return Group(); }
};

class Exception {
  public:
    static void dontPrint() {}
};
class FileIException : public Exception {};

}  // namespace H5

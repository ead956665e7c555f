// Stand-in for the HDF5 C++ header: the reference's beam/kernel headers name
// these types only in declarations of file-I/O members that the harness never
// calls.
#pragma once
namespace H5 {
class CompType {};
class Group {};
class DataSpace {};
}  // namespace H5

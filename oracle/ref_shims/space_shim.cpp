// Project-written stand-ins for the HDF5 entry points that libvvhd/src/TSpace.cpp names
// (declared in hdf5_stub/hdf5.h) and for the members of Space whose translation units need
// HDF5 (TSpace_save_hdf.cpp, TSpace_load_hdf.cpp, TSpace_load_v13.cpp).  TSpace.cpp itself
// is compiled unmodified, so Space's constructor, calc_forces and zero_forces are the
// reference's own.  Snapshot I/O is not part of the oracle: these report failure.
// TEST INFRASTRUCTURE ONLY.
#include <stdexcept>
#include <string>

#include "TSpace.hpp"
#include "hdf5.h"

herr_t H5Eset_auto(hid_t, void*, void*) { return -1; }
htri_t H5Fis_hdf5(const char*) { return -1; }
hid_t H5Fopen(const char*, unsigned, hid_t) { return -1; }
hid_t H5Fcreate(const char*, unsigned, hid_t, hid_t) { return -1; }
herr_t H5Fclose(hid_t) { return -1; }

void h5_throw(std::string fn, std::string arg) { throw std::runtime_error(fn + " " + arg + ": no HDF5 in the oracle"); }

void Space::save_hdf(int64_t) { throw std::runtime_error("Space::save_hdf: no HDF5 in the oracle"); }
void Space::load_hdf(int64_t, metainfo_t*) { throw std::runtime_error("Space::load_hdf: no HDF5 in the oracle"); }
void Space::load_v13(const char*) { throw std::runtime_error("Space::load_v13: not in the oracle"); }

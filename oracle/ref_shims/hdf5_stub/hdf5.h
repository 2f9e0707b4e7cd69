// Project-written stand-in for the HDF5 header, declaring only what libvvhd/src/TSpace.cpp
// and libvvhd/headers/vvhdf.h name, so that TSpace.cpp compiles unmodified for the oracle.
// The functions are defined in space_shim.cpp and report failure if called (snapshot I/O
// is not part of the oracle).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include <cstdint>

typedef int64_t hid_t;
typedef int herr_t;
typedef int htri_t;
typedef unsigned long long hsize_t;

#define H5E_DEFAULT 0
#define H5P_DEFAULT 0
#define H5F_ACC_RDONLY 0u
#define H5F_ACC_TRUNC 2u

herr_t H5Eset_auto(hid_t estack, void* func, void* client_data);
htri_t H5Fis_hdf5(const char* name);
hid_t H5Fopen(const char* name, unsigned flags, hid_t fapl);
hid_t H5Fcreate(const char* name, unsigned flags, hid_t fcpl, hid_t fapl);
herr_t H5Fclose(hid_t fid);

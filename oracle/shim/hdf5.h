/* Oracle test infrastructure: a type-only stand-in for the HDF5 C API header.
 *
 * The reference's GridObj_ops_io.cpp includes hdf5.h unconditionally (through
 * inc/hdf5luma.h) for its HDF5 writer; the oracle build compiles that file for
 * its ASCII writers (io_lite, io_restart) and never calls the HDF5 writer.
 * Everything here only has to compile: the handle types, the constants the
 * writer names, and do-nothing functions that accept any arguments. */
#ifndef LUMA_ORACLE_HDF5_SHIM_H
#define LUMA_ORACLE_HDF5_SHIM_H
#include <cstdint>

typedef int64_t hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;

enum { H5P_DEFAULT = 0, H5E_DEFAULT = 0, H5P_FILE_ACCESS = 1, H5P_DATASET_XFER = 2,
       H5T_NATIVE_INT = 3, H5T_NATIVE_DOUBLE = 4, H5F_ACC_TRUNC = 5, H5F_ACC_RDWR = 6,
       H5S_SELECT_SET = 7, H5FD_MPIO_COLLECTIVE = 8 };

#define LUMA_H5_STUB(name) \
    template <class... T> static inline hid_t name(T...) { return 0; }
LUMA_H5_STUB(H5Dcreate)
LUMA_H5_STUB(H5Dclose)
LUMA_H5_STUB(H5Dwrite)
LUMA_H5_STUB(H5Acreate)
LUMA_H5_STUB(H5Awrite)
LUMA_H5_STUB(H5Aclose)
LUMA_H5_STUB(H5Screate_simple)
LUMA_H5_STUB(H5Sclose)
LUMA_H5_STUB(H5Sselect_none)
LUMA_H5_STUB(H5Sselect_hyperslab)
LUMA_H5_STUB(H5Pcreate)
LUMA_H5_STUB(H5Pclose)
LUMA_H5_STUB(H5Pset_fapl_mpio)
LUMA_H5_STUB(H5Pset_dxpl_mpio)
LUMA_H5_STUB(H5Fcreate)
LUMA_H5_STUB(H5Fopen)
LUMA_H5_STUB(H5Fclose)
LUMA_H5_STUB(H5Gcreate)
LUMA_H5_STUB(H5Gclose)
LUMA_H5_STUB(H5Eset_auto)
LUMA_H5_STUB(H5Eprint)
#undef LUMA_H5_STUB

#endif

/* Serial stand-in for <hdf5.h>, used only so that the reference's
 * h5part_writer.cc compiles into the 1D oracle build for its write_csv.
 * Types and declarations; the definitions in ref/h5_stub.cc abort if they
 * are ever called (write_csv calls none of them). */
#ifndef ORACLE_STUB_HDF5_H
#define ORACLE_STUB_HDF5_H
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef enum { H5F_SCOPE_LOCAL = 0, H5F_SCOPE_GLOBAL = 1 } H5F_scope_t;
herr_t H5Fclose(hid_t);
herr_t H5Gclose(hid_t);
herr_t H5Fflush(hid_t, H5F_scope_t);
#endif

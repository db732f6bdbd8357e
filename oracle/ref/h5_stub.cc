// h5_stub.cc -- project-written definitions behind ref/stub/hdf5.h and the
// reference's hdf5calls.h declarations, so that h5part_writer.cc links into
// the 1D oracle build.  The build exercises only write_csv
// (h5part_writer.cc:448-490), which uses none of these; each one aborts.
#include <cstdio>
#include <cstdlib>
#include <hdf5.h>
#include "hdf5calls.h"

static void no_hdf5(const char *f) {
  std::fprintf(stderr, "%s: HDF5 is not part of the oracle build\n", f);
  std::abort();
}
herr_t H5Fclose(hid_t) { no_hdf5("H5Fclose"); return -1; }
herr_t H5Gclose(hid_t) { no_hdf5("H5Gclose"); return -1; }
herr_t H5Fflush(hid_t, H5F_scope_t) { no_hdf5("H5Fflush"); return -1; }
hid_t GH5_fopen_serial(const char *, char) { no_hdf5("GH5_fopen_serial"); return -1; }
hid_t GH5_gopen(hid_t, const char *, char) { no_hdf5("GH5_gopen"); return -1; }
herr_t GH5_WriteS(hid_t, const char *, int *, void *, int, int, const int) { no_hdf5("GH5_WriteS"); return -1; }

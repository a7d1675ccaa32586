/*
 * muto_io.h -- C entry points of the host reconstruction library
 * (lib/libmuto_facade.so, the C++ classes over include/muto_gb300.h).
 *
 * muto_read_muon_data replaces MutoFile::getMuonData (src/MutoFile.cpp:19-82
 * with the per-record line fit of :248-304): records of 2*nz+2 values
 * {ein, x0, y0, ..., x_{nz-1}, y_{nz-1}, eout} (float32 when precision is 4,
 * float64 when 8); records holding a NaN are skipped; layers 0..n_middle-1
 * give the incoming line and n_middle..nz-1 the outgoing one, each the
 * principal axis of its hits oriented with d_z > 0, with pin on layer
 * n_middle-1 and pout on layer n_middle.
 * Call with out == NULL to get the number of tracks in *n_out (the records
 * without a NaN; nothing is fitted); otherwise at most cap tracks are
 * written and *n_out is the number written.  Records are read 2^20 at a time
 * and fitted in parallel (OpenMP threads of the calling process); the result
 * does not depend on the thread count.  Files are opened by name (a file
 * that cannot be opened is reported and skipped, as the reference does).
 */
#ifndef MUTO_IO_H
#define MUTO_IO_H

#include <stdint.h>

#include "muto_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int muto_read_muon_data(const char* const* files, int n_files, const double* z_layers, int nz, int n_middle,
                        int precision, muto_ray* out, uint64_t cap, uint64_t* n_out);

#ifdef __cplusplus
}
#endif

#endif /* MUTO_IO_H */

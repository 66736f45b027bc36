#ifndef DMG_IO_H
#define DMG_IO_H
/**
 * Global-order input and output of a distributed array.
 *
 * The reference writes and reads distributed arrays through an MPI-IO file
 * view (reshape.c:137-147 makeGlobalIndex, reshape.c:158-172 expandIOType,
 * reshape.c:494-521 makeIOType; used by fftw_bench.c:26-100 writeFile /
 * readFile, fftw_test.c:30-180, plan_compare.c:50-200): each rank's view
 * places its local elements at their global C-order positions, so the file
 * holds the global array in C order (last dimension fastest) whatever the
 * decomposition.  On the virtual grid the whole array is one device buffer
 * (rank r at element r * pitch), so the same file comes from one permutation
 * kernel into a "global" layout followed by a device-to-host copy and a
 * write; reading runs the inverse.  These entry points have no counterpart
 * in the reference's API (which exposes the MPI datatype instead).
 */
#include "reshape.h"

#ifdef __cplusplus
extern "C" {
#endif

/** A decomposition with every element on rank 0 in packed C order: its
 * buffer is the global array, element (x0, x1, ...) at its C-order linear
 * index. */
Decomp dmg_makeGlobalDecomp(MPI_Comm comm, int ndim, const int *L);

/** Device to device: global[linear(x)] = the element at x of the array in
 * decomposition d (rank r's buffer at element r * extent64(d) of src). */
int dmg_io_gather(Decomp d, MPI_Datatype type, const void *src, void *global, void *stream);
/** Device to device, the inverse: every element d holds is set from global. */
int dmg_io_scatter(Decomp d, MPI_Datatype type, const void *global, void *dst, void *stream);

/** Write the array (device buffer in decomposition d) to a file in global
 * C order, as writeFile (fftw_bench.c:26-63) does through makeIOType.  Uses
 * a temporary device buffer and a host buffer of the whole array; waits
 * for the stream. */
int dmg_io_write_file(const char *path, Decomp d, MPI_Datatype type, const void *src, void *stream);
/** Read a global C-order file into the device buffer of decomposition d, as
 * readFile (fftw_bench.c:64-100). */
int dmg_io_read_file(const char *path, Decomp d, MPI_Datatype type, void *dst, void *stream);

/** The file view makeIOType builds for one rank: for each element the rank
 * holds, in the order writeFile visits them (global coordinates in C order),
 * its file position (C-order linear index) and its offset in the rank's
 * buffer (getOffset).  Returns the count (at most max written). */
long long dmg_io_view(Decomp d, int rank, long long *file_off, long long *mem_off, long long max);

#ifdef __cplusplus
}
#endif
#endif

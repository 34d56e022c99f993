/* fair_io.h -- the file formats of the reference's driver (host-only).
 *
 *  - Matrix files of store_matrix / read_csr_matrix
 *    (system_generation.f90:595-665): a gfortran unformatted sequential file
 *    of six records, m, n, nnz (4-byte integers), vA (nnz FP64), JA (nnz
 *    4-byte, 1-based), IA (m+1 4-byte, IA(0) = 0), each record framed by
 *    4-byte length markers; a record longer than 2^31-9 bytes is written as
 *    gfortran's subrecords (negative markers flag the continued parts).
 *  - Input files of read_data (system_generation.f90:494-539), ordering files
 *    of read_ordering (:567-593) and reference solutions of read_ref
 *    (:541-565), read with Fortran list-directed rules: every READ starts on
 *    a new line, takes its items across lines as needed, and drops the rest
 *    of its last line; D exponents are accepted.
 *  - Solution files written like main.f90:354-358 (one value per line,
 *    list-directed layout, 17 significant digits).
 * All functions return the status codes of fair_gpu.h; a malformed file is
 * FAIR_ERR_ARG with the reason in fair_last_error_detail().
 */
#ifndef FAIR_IO_H
#define FAIR_IO_H

#include "fair_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Matrix files (host arrays). */
int fair_write_csr_file(const char *path, int32_t m, int32_t n, int32_t nnz, const double *vA,
                        const int32_t *JA, const int32_t *IA);
int fair_read_csr_file_sizes(const char *path, int32_t *m, int32_t *n, int32_t *nnz);
int fair_read_csr_file(const char *path, double *vA, int32_t *JA, int32_t *IA);
/* store_matrix / read_csr_matrix on a handle (the matrix goes through the
 * host; nnz must fit the file's 4-byte integers). */
int fair_store_matrix(fair_csr h, const char *path);
int fair_read_csr_matrix(fair_csr h, const char *path);

/* read_data: sizes first, then the data into caller buffers (theta: nth
 * entries, converted from degrees to radians as the reference does; T: nth*p
 * transmission values). dat->theta is set to theta. The reference's stops
 * ("Angle vector has the wrong length, nth is incorrect.", "Data has the
 * wrong size, or p and nth are incorrect.") are FAIR_ERR_ARG with that text. */
int fair_read_data_sizes(const char *path, int32_t *n, int32_t *p, int32_t *nth);
int fair_read_data(const char *path, fair_data *dat, double *theta, double *T);

/* read_ordering: *len receives the count; order (capacity entries, may be
 * NULL to query the count) the 1-based row numbers. */
int fair_read_ordering(const char *path, int32_t *len, int32_t *order, int32_t capacity);
/* read_ref: n values, one per line. */
int fair_read_ref(const char *path, int64_t n, double *xref);

/* One value per line, as main.f90 writes sol.txt and errorgauge.txt. */
int fair_write_values(const char *path, const double *x, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* FAIR_IO_H */

/* MPAS-format files without HDF5: a reader and writer of the netCDF classic
 * formats (CDF-1, CDF-2 "64-bit offset", CDF-5 "64-bit data"), the formats
 * MPAS mesh and history files are commonly distributed in.
 *
 * Replaces, for files in those formats, the reference's HDF5 I/O layer:
 *   - mesh connectivity read by definition::read_entities
 *     (mpasoflecsi/specialization/definition.hh:1055-1106, via
 *     mpasoflecsi/io/io_hdf5.hh read_connectivity_2D),
 *   - mesh and ocean fields read by read_mesh_fields / read_ocean_mesh_fields
 *     (mpasoflecsi/tasks/io.cc:14-158, mpasoflecsi/io/helpers.hh helper1d /
 *     helper2d ::read),
 *   - history output: mesh_output_init (mpasoflecsi/tasks/io.cc:160-247) and
 *     helper1d::write_timestep (mpasoflecsi/io/helpers.hh:127-151), which
 *     write one record per output time along the Time dimension.
 * HDF5-based netCDF-4 files (what the reference opens with H5Fopen) need
 * libhdf5, which libmpaso does not link; `nccopy -k cdf5 in.nc out.nc`
 * converts them.  Host code only: no GPU needed.
 *
 * All functions return MPASO_OK or an MPASO_ERR_* code (mpaso_mesh.h); the
 * message is in mpaso_last_error().  A handle is used by one thread at a time.
 */
#ifndef MPASO_IO_H
#define MPASO_IO_H

#include <stdint.h>

#include "mpaso_mesh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* external types (the netCDF nc_type codes) */
#define MPASO_NC_BYTE 1
#define MPASO_NC_CHAR 2
#define MPASO_NC_SHORT 3
#define MPASO_NC_INT 4
#define MPASO_NC_FLOAT 5
#define MPASO_NC_DOUBLE 6
#define MPASO_NC_INT64 10 /* CDF-5 only */

typedef struct mpaso_nc_s *mpaso_nc;

/* Open an existing file; writable = 1 allows appending records (mpaso_nc_put_rec). */
int mpaso_nc_open(const char *path, int32_t writable, mpaso_nc *out);
/* Create (truncate) a file in define mode; version 1, 2 or 5. */
int mpaso_nc_create(const char *path, int32_t version, mpaso_nc *out);
/* Flush (header record count included) and close. */
int mpaso_nc_close(mpaso_nc f);

/* Define mode (after create).  len = 0 defines the record (unlimited)
 * dimension, which must then be a variable's first dimension.  Attribute
 * values are given in their own type (char text, int32, double, ...). */
int mpaso_nc_def_dim(mpaso_nc f, const char *name, int64_t len);
int mpaso_nc_def_var(mpaso_nc f, const char *name, int32_t type, int32_t ndims, const char *const *dims);
int mpaso_nc_put_att(mpaso_nc f, const char *var /* NULL: global */, const char *name, int32_t type,
                     int64_t n, const void *values);
/* Leave define mode: lays the variables out and writes the header. */
int mpaso_nc_enddef(mpaso_nc f);

/* Data.  mem_type is the type of the caller's buffer (numeric types convert
 * to and from one another; CHAR only to CHAR).  put_var / get_var move a whole
 * fixed-size variable (get_var of a record variable reads every record);
 * put_rec / get_rec move record `rec` of a record variable (put_rec may append
 * one past the last record). */
int mpaso_nc_put_var(mpaso_nc f, const char *name, int32_t mem_type, const void *data);
int mpaso_nc_put_rec(mpaso_nc f, const char *name, int64_t rec, int32_t mem_type, const void *data);
int mpaso_nc_get_var(mpaso_nc f, const char *name, int32_t mem_type, void *out);
int mpaso_nc_get_rec(mpaso_nc f, const char *name, int64_t rec, int32_t mem_type, void *out);

/* Queries.  Shapes report the record dimension as the current record count.
 * Names are copied NUL-terminated into buf (buflen bytes). */
int mpaso_nc_inq(mpaso_nc f, int32_t *version, int64_t *numrecs, int32_t *ndims, int32_t *nvars,
                 int32_t *ngatts);
int mpaso_nc_inq_dim(mpaso_nc f, const char *name, int64_t *len);
int mpaso_nc_dim_name(mpaso_nc f, int32_t id, char *buf, int32_t buflen, int64_t *len);
int mpaso_nc_var_name(mpaso_nc f, int32_t id, char *buf, int32_t buflen);
int mpaso_nc_inq_var(mpaso_nc f, const char *name, int32_t *type, int32_t *ndims, int64_t *shape /* [8] */,
                     int32_t *is_record);
int mpaso_nc_var_dim_name(mpaso_nc f, const char *var, int32_t i, char *buf, int32_t buflen);
/* Attribute: *type and *n (element count) always; the values too when out is
 * not NULL and cap_bytes holds them (in the attribute's own type). */
int mpaso_nc_get_att(mpaso_nc f, const char *var /* NULL: global */, const char *name, int32_t *type,
                     int64_t *n, void *out, int64_t cap_bytes);
int mpaso_nc_att_name(mpaso_nc f, const char *var /* NULL: global */, int32_t id, char *buf, int32_t buflen);

#ifdef __cplusplus
}
#endif
#endif

/*
 * mpaso_mesh.h -- host-side mesh services of libmpaso (no GPU needed).
 *
 * The reference reads MPAS meshes from HDF5 files (mpasoflecsi/specialization/
 * definition.hh:1055-1106) and computes the FCT / del2 static coefficients on
 * the host once (apps/ocean/tasks/init_functions.cc:18-447).  libmpaso does not
 * link HDF5, so it generates the same MPAS mesh datasets in memory:
 *
 *   - a quasi-uniform sphere, the Voronoi dual of a recursively bisected
 *     icosahedron (10*4^level + 2 cells);
 *   - a doubly periodic planar hexagonal mesh (nx*ny cells).
 *
 * Every dataset is exposed under its MPAS name with the MPAS file conventions:
 * connectivity is int32, 1-based, padded with 0 up to maxEdges (8) /
 * maxEdges2 (16) / vertexDegree (3) columns; real fields are float64.
 *
 * All functions return 0 on success and a nonzero MPASO_ERR_* code on failure;
 * mpaso_last_error() returns the calling thread's last message.
 */
#ifndef MPASO_MESH_H
#define MPASO_MESH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPASO_OK 0
#define MPASO_ERR_ARG 1       /* bad argument (null pointer, size out of range) */
#define MPASO_ERR_MESH 2      /* inconsistent mesh / connectivity */
#define MPASO_ERR_CUDA 3      /* CUDA runtime error */
#define MPASO_ERR_ALLOC 4     /* allocation failure (host or device) */
#define MPASO_ERR_NOTFOUND 5  /* unknown dataset name */
#define MPASO_ERR_TIMEOUT 6   /* reserved: a bounded device-side wait gave up (no kernel waits today) */
#define MPASO_ERR_NUMERIC 7   /* non-finite value found (mpaso_state_check_finite) */
#define MPASO_ERR_NODEVICE 8  /* no CUDA device available */
#define MPASO_ERR_IO 9        /* file open / read / write failure or malformed file */

#define MPASO_DTYPE_INT32 0
#define MPASO_DTYPE_FLOAT64 1

typedef struct mpaso_genmesh_s *mpaso_genmesh;

/* Thread-local text of the last error raised by any libmpaso call. */
const char *mpaso_last_error(void);

/* Sphere of radius `radius` (m): dual of a level-`level` icosahedral
 * subdivision, 0 <= level <= 10.  A fixed generic rotation is applied so that
 * no generator lies on a coordinate plane. f = 2*omega*sin(lat). */
int mpaso_genmesh_icosa(int level, double radius, double omega, mpaso_genmesh *out);

/* Doubly periodic hexagonal mesh with nx columns, ny rows (ny even, nx,ny >= 4)
 * and cell-centre spacing dc (m); f-plane Coriolis f0 everywhere. */
int mpaso_genmesh_hex(int nx, int ny, double dc, double f0, mpaso_genmesh *out);

/* Renumber a generated mesh along a space-filling curve (cells by curve key,
 * edges and vertices by their lowest new cell), keeping every MPAS ordering
 * convention.  Produces a new handle; `perm_cell[new] = old` etc. if non-null. */
int mpaso_genmesh_reorder_sfc(mpaso_genmesh in, mpaso_genmesh *out,
                              int32_t *perm_cell, int32_t *perm_edge, int32_t *perm_vertex);

/* dims[0..2] = nCells, nEdges, nVertices; flags[0] = 1 on a sphere,
 * geom[0..2] = sphere radius, periodic x-extent, periodic y-extent. */
int mpaso_genmesh_dims(mpaso_genmesh m, int64_t dims[3], int32_t flags[1], double geom[3]);

/* Shape and element type of a named dataset. */
int mpaso_genmesh_field(mpaso_genmesh m, const char *name, int32_t *dtype,
                        int64_t *rows, int64_t *cols);

/* Copy a named dataset (rows*cols elements) into dst. */
int mpaso_genmesh_copy(mpaso_genmesh m, const char *name, void *dst);

/* Names of all datasets, separated by ','. */
const char *mpaso_genmesh_names(void);

void mpaso_genmesh_free(mpaso_genmesh m);

/* ------------------------------------------------------------------------
 * FCT / del2 static coefficients (host), the setup of
 * apps/ocean/tasks/init_functions.cc:18-447 as apps/ocean/initialize.cc:
 * 391-400 runs it: maxLevelEdgeTop, meshScalingDel2, edgeSignOnCell,
 * derivTwo (second-derivative least-squares fit on the tangent plane),
 * advCellsForEdge / advCoef / advCoef_3rd, highOrderAdvMask.
 * On the sphere the results equal the reference's bit for bit.  The
 * reference has no planar branch (init_functions.cc:198-200, 282-283,
 * 321-322 are empty); on_sphere = 0 fits the same polynomial in plane
 * coordinates with minimum-image offsets on a periodic domain.
 * Connectivity is FleCSI's 0-based CRS in file order (as in mpaso_mesh_desc).
 * ---------------------------------------------------------------------- */
typedef struct {
  int64_t nCells, nEdges, nVertices;
  const int64_t *c2e_off, *c2c_off, *e2v_off;
  const int32_t *c2e, *c2c, *e2v;
  const double *dcEdge, *dvEdge;
  const double *xCell, *yCell, *zCell, *xVertex, *yVertex, *zVertex;
  const double *meshDensity;
  int32_t on_sphere;
  double Lx, Ly;               /* planar periodic extents (0 = not periodic) */
  int32_t nlev;
  const int32_t *maxLevelCell; /* [nC] */
  const int32_t *boundaryCell; /* [nC][nlev]; NULL = no boundary cells */
} mpaso_fct_setup_in;

typedef struct {
  int32_t *maxLevelEdgeTop;  /* [nE] */
  double *meshScalingDel2;   /* [nE] */
  double *edgeSignOnCell;    /* [nC][8] */
  double *derivTwo;          /* [nE][16][2] */
  int32_t *nAdvCellsForEdge; /* [nE] */
  int32_t *advCellsForEdge;  /* [nE][16] */
  int32_t *highOrderAdvMask; /* [nE][nlev] */
  double *advCoef, *advCoef_3rd; /* [nE][16] */
} mpaso_fct_setup_out;

int mpaso_fct_setup(const mpaso_fct_setup_in *in, mpaso_fct_setup_out *out);

/* The same setup computed on GPU `device` (host arrays in and out; the call
 * returns when the outputs are written).  No counterpart in the reference,
 * which runs it on the host at start-up (apps/ocean/initialize.cc:88-102).
 * One thread per cell fits the second-derivative polynomial and one per edge
 * assembles the advection stencil; offsets and indices are validated on the
 * host first.  Integer outputs equal mpaso_fct_setup's exactly; derivTwo and
 * the advection coefficients agree with it to the last-place differences of
 * CUDA's acos / asin / sin / cos / atan2 against the C library's.  For meshes
 * of many cells, or ensembles, where the host setup costs ~10 us per cell. */
int mpaso_fct_setup_device(const mpaso_fct_setup_in *in, mpaso_fct_setup_out *out, int32_t device);

/* The device setup of n meshes in one call (one allocation, one stream):
 * ins[i] -> outs[i].  An error names the first failing member. */
int mpaso_fct_setup_device_many(const mpaso_fct_setup_in *ins, mpaso_fct_setup_out *outs, int32_t n,
                                int32_t device);

#ifdef __cplusplus
}
#endif
#endif

/*
 * fcgpu_meshgen.h -- synthetic-input side of libfcgpu.so.
 *
 * The reference reads its meshes from polyMesh files and computes their geometry in
 * mesh_geometry (src/mesh_geometry_and_topology.f90:310-1222).  These entry points
 * produce the same arrays for a jittered hexahedral mesh of the unit cube, so that
 * large cases (up to 256^3 cells) can be generated in memory with a seeded,
 * counter-based random number generator.  All index outputs are 1-based.
 */
#ifndef FCGPU_MESHGEN_H
#define FCGPU_MESHGEN_H

#ifdef __cplusplus
extern "C" {
#endif

/* Sizes of the N x N x N hex mesh (no reference counterpart). */
int fcg_hex_mesh_sizes(int N, int *numNodes, int *numCells, int *numFaces, int *numInnerFaces);

/* Builds the N^3 hex mesh of the unit cube (no reference counterpart; it stands in
 * for a polyMesh on disk).  Interior vertices are displaced by i.i.d.
 * U(-jitter*h, jitter*h) per axis; boundary vertices stay fixed.  Faces follow the
 * OpenFOAM order: inner faces sorted by owner then neighbour, then the boundary
 * faces, symmetry patches (x=1, y=0, y=1, z=0, z=1) first and the wall patch x=0
 * last, each face ordered so that its area vector points out of its owner.
 * Outputs: x,y,z[numNodes]; face_ptr[numFaces+1] (0-based offsets, 4 nodes a face);
 * face_nodes[4*numFaces] (1-based); owner[numFaces]; neighbour[numInnerFaces];
 * patches[4] = {nsym, iSymmetryFacesStart, nwal, iWallFacesStart}. */
int fcg_hex_mesh_build(int N, double jitter, unsigned long long seed, double *x, double *y,
                       double *z, int *face_ptr, int *face_nodes, int *owner, int *neighbour,
                       int *patches);

/* Geometry of mesh_geometry (mesh_geometry_and_topology.f90:859-1079): face area
 * vectors by triangle fans from the first node, arithmetic-mean face centres,
 * divergence-theorem volumes, Nurnberg centroids and the interpolation factor through
 * the plane of the first three face nodes.  Same expressions in the same order as
 * the Fortran loops (bit-identical results), computed per cell in parallel. */
int fcg_mesh_geometry(int numNodes, const double *x, const double *y, const double *z,
                      int numCells, int numFaces, int numInnerFaces, const int *face_ptr,
                      const int *face_nodes, const int *owner, const int *neighbour,
                      double *arx, double *ary, double *arz, double *xf, double *yf,
                      double *zf, double *xc, double *yc, double *zc, double *vol,
                      double *facint);

/* Fills out[i] = lo + (hi-lo) * U_i, U_i in [0,1) from a counter-based generator
 * keyed by (seed, stream, i): the same numbers on every machine and thread count. */
int fcg_uniform_fill(unsigned long long seed, unsigned long long stream, long long count,
                     double lo, double hi, double *out);

#ifdef __cplusplus
}
#endif
#endif /* FCGPU_MESHGEN_H */

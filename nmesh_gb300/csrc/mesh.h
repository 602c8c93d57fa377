// mesh.h -- host-side packed mesh shared by the mesh packer (mesh.cpp) and
// the device context (nmg.cu).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace nmg {
// a patch of a generated mesh: a Cartesian box or an outer cubed-sphere
// patch (coordtrans_CubedSphere.c with constant sigma)
struct Patch {
  double bbox[6];
  bool cubed = false;  // outer cubed-sphere patch (else Cartesian box)
  bool shell = false;  // ... with a curved inner surface too (radius s0)
  int dom = 0;         // cubed-sphere domain 0..5
  double xc[3] = {0, 0, 0};
  double s0 = 0, s1 = 0;  // inner flat distance and outer sphere radius
};
}  // namespace nmg

struct nmg_mesh {
  int n = 0;        // LGL nodes per direction
  int64_t nelem = 0;
  std::vector<int32_t> pat;    // [E] patch index
  std::vector<double> bbox;    // [E][6] bbox in patch coordinates
  std::vector<int32_t> curvi;  // [E] 1 if the patch map is not Cartesian
  std::vector<double> xyz;     // [E][3][np]
  std::vector<double> dXdx;    // [E][9][np] dX^a/dx^i (identity if Cartesian)
  std::vector<int32_t> nb;     // [E][6] neighbour element, -1 on outer faces
  std::vector<int32_t> code;   // [E][6] neighbour face | orientation << 3
  std::vector<double> x, w, D; // LGL points, quadrature weights, D[i*n+j]
  std::vector<double> xu;      // equally spaced points (finite-volume elements)
  std::vector<int32_t> fv;     // [E] 1: finite-volume element on equally
                               // spaced points; empty: all DG on LGL points
  std::vector<nmg::Patch> patches;  // patch maps of a generated mesh (empty
                                    // for a described one)
  std::vector<std::string> names;   // [E] the reference's element names
                                    // "<patch>_<octree digits>" (generated meshes)
  int ndiv = 0;                     // > 0: patches split into ndiv^3 equal elements
  std::vector<int32_t> level;       // [E] refinement level (generated meshes)
  std::vector<int32_t> ixyz;        // [E][3] integer position at that level
  // Non-conforming faces (a level jump between neighbours): per such face
  // (element, face) and, per face node, the list of contributions (source
  // element, source face, the node's position in the source face's
  // in-plane coordinates in [-1,1]); the trace is the average of the
  // contributions' interpolated values.
  std::vector<int32_t> hface;       // [H][2]
  std::vector<int32_t> hoff;        // [H*n*n + 1]
  std::vector<int32_t> hsrc;        // [C][2]
  std::vector<double> hpos;         // [C][2]
};

// face-table code bit: the neighbour has the other point type (DG / FV), its
// trace is interpolated onto this face's points
constexpr int NMG_CODE_MIXED = 64;
// face-table bit: the face is non-conforming (neighbours of another level),
// its trace is interpolated from the listed neighbour faces
constexpr int NMG_CODE_HANG = 128;

namespace nmg {
// LGL nodes/weights and differentiation matrix (Legendre.c / Lagrange.c)
void lgl_basis(int n, double *x, double *w, double *D);
// equally spaced points with trapezoid weights (uniform_x_wTrapez,
// Legendre.c:626-719) and the Lagrange D matrix on them
void uniform_basis(int n, double *x, double *w, double *D);
// in-plane node (a, b) of face f -> volume index i + n*(j + n*k)
inline int face_node(int n, int f, int a, int b) {
  int d = f >> 1, p = (f & 1) * (n - 1);
  if (d == 0) return p + n * (a + n * b);
  if (d == 1) return a + n * (p + n * b);
  return a + n * (b + n * p);
}
// coordinates [3][np] and dX^a/dx^i [9][np] of element e on LGL points
// (uniform = false) or equally spaced points; false if the element's patch
// map is not known (a described curvilinear element)
bool element_geometry(const nmg_mesh &m, int64_t e, bool uniform, double *xyz, double *dXdx);
// dX^a/dx^i [3][9][np] of element e at the midpoints between its equally
// spaced points: block d holds, at node (i, j, k), the values at the
// midpoint to the right of that node in direction d (the last plane of each
// direction is unused, zero); false if the element's map is unknown
bool element_midpoint_dXdx(const nmg_mesh &m, int64_t e, double *dXdxm);
// apply a dihedral orientation code to an in-plane index pair
inline void orient_map(int n, int o, int a, int b, int *a2, int *b2) {
  int s = o & 1, fa = (o >> 1) & 1, fb = (o >> 2) & 1;
  int aa = s ? b : a, bb = s ? a : b;
  *a2 = fa ? n - 1 - aa : aa;
  *b2 = fb ? n - 1 - bb : bb;
}
// build neighbour/orientation table from coordinates (or an explicit
// node table); returns an error string or empty on success
std::string pack_faces(nmg_mesh &m, const int64_t *nbnode, const double period[3]);
}  // namespace nmg

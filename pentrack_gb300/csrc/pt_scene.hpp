/*
 * pt_scene.hpp -- host-side preparation of the device scene.
 *
 * Setup-time work that the reference does in TGeometry / TTriangleMesh::ReadFile
 * (AABB tree build, src/trianglemesh.cpp:120-121) and in the TabField3
 * constructor (derivative tables and cell coefficients, src/field_3d.cpp:336-484),
 * re-laid-out for the GPU: a depth-first flattened BVH with skip indices and
 * per-node cubic-Hermite data instead of 64 coefficients per cell.
 */
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include "../../include/pentrack_gpu.h"

namespace pth {

struct HostTri { double a[3], b[3], c[3], n[3]; int solid; int pad; };
struct HostNode { float lo[3], hi[3]; int skip; int leaf; };

/* Builds the flattened BVH over the scene's triangles; `tris` is reordered so
 * every leaf covers a contiguous range of at most 4 triangles. */
void build_bvh(std::vector<HostTri> &tris, std::vector<HostNode> &nodes);

/* ALGLIB spline1dgriddiffcubic with parabolically terminated ends
 * (alglib-3.15.0/cpp/src/interpolation.cpp:26709-26880), as TabField3::CalcDerivs uses it. */
void spline_derivs(int n, const double *x, const double *y, double *d);

/* Per-node Hermite data (f, fx, fy, fz, fxy, fxz, fyz, fxyz) of one [ix][iy][iz]
 * table, with the derivative tables built in TabField3::PreInterpol's order
 * (src/field_3d.cpp:374-381).  out[node*stride + comp*8 + k]. */
void hermite_nodes(const std::vector<double> ax[3], const double *tab, int comp, int stride, std::vector<double> &out);

/* TabField's bicubic spline data (ALGLIB spline2dbuildbicubicv,
 * alglib-3.15.0/cpp/src/interpolation.cpp:44925-45080 and 46791-46880) of
 * one [ir][iz] table: per node f, df/dr, df/dz, d2f/drdz, each slope as
 * spline1ddiff returns it from the parabolically terminated cubic spline
 * along that axis (d2f/drdz: along r of the d/dz table).
 * out[(ir*nz + iz)*stride + comp*4 + k]. */
void bicubic_nodes(const std::vector<double> &r, const std::vector<double> &z, const double *tab, int comp, int stride,
                   std::vector<double> &out);

/* FP32 node table from per-node Hermite data (stride ncomp*8): per node and
 * component 9 floats -- the value as FP32 high part and FP32 rounding of the
 * rest, then fx, fy, fz, fxy, fxz, fyz, fxyz rounded to FP32 -- with the
 * node record padded to a multiple of 4 floats.  Returns the floats per node. */
int node_table32(const std::vector<double> &nodes, int ncomp, std::vector<float> &out);

/* Harmonic expansion (HarmonicExpandedBField, src/harmonicfields.cpp:50-829)
 * written as one scalar polynomial Phi with B = grad Phi.  Each G(l,m) adds
 * G * (l)! 2^|m| / (l+1+|m|)! * r^(l+1) P_(l+1)^|m|(cos theta) * {cos|m|phi (m>=0), sin|m|phi (m<0)}
 * (Legendre functions without the Condon-Shortley phase).  Exponents are
 * packed i | j<<4 | k<<8. */
bool harmonic_polynomial(int n, const int32_t *l, const int32_t *m, const double *g, std::vector<double> &coef,
                         std::vector<int> &expo, std::string &err);

} // namespace pth

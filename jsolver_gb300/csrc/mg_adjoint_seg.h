// mg_adjoint_seg.h — what the adjoint's single-block segments need: the adjoint arrays
// of a level, the level tables and a segment of tape operators, laid out in device
// memory by mg_adjoint.cu and executed by mg_adjoint_kernels.cu.
#pragma once

#include <cuda_runtime.h>

#include "mg_common.cuh"

namespace jmg {

// adjoint arrays of one level: pb = adjoint of phi, rb = adjoint of rhs, T = scratch,
// gacc / gwx / gwy / gwz = adjoints of A_cc and of the x / y / z face couplings (gwz in 3D),
// gxll .. gxrr = adjoints of the diagonal couplings of the 9-point stencil (2D with D_xy);
// absent arrays are nullptr
struct AdjLvl {
  double *pb, *rb, *T, *gacc, *gwx, *gwy, *gwz;
  double *gxll, *gxrl, *gxlr, *gxrr;
};

enum { kAdjOpSweep = 0, kAdjOpRestrict = 1, kAdjOpProlong = 2 };

// one operator of the tape with its phi states resolved to addresses: before = phi the
// operator read, after = where the forward stores phi after it (sweeps, prolongations)
struct AdjSegOp {
  int kind, lev;
  const double* before;
  double* after;
};

constexpr int kMaxSegOps = 112;  // the struct stays under the 4 KB of a kernel parameter
struct AdjSeg {
  int n, pad;
  AdjSegOp op[kMaxSegOps];
};

struct AdjTables {
  LvlTable<double> lv;
  AdjLvl g[kMaxLevels];
};

void adj_store_tables(const AdjTables& t, AdjTables* dst, cudaStream_t s);
void adj_store_seg(const AdjSeg& g, AdjSeg* dst, cudaStream_t s);
void adj_seg_fwd(int dim, const AdjTables* t, const AdjSeg* g, bool snapshots, int diag, cudaStream_t s);
void adj_seg_rev(int dim, const AdjTables* t, const AdjSeg* g, int diag, cudaStream_t s);

}  // namespace jmg

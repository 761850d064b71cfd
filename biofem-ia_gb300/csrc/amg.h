/*
 * Smoothed-aggregation algebraic multigrid for the assembled tangent (3x3
 * block rows), used as the preconditioner of the device Newton solve.
 *
 * Symbolic part (host, once per mesh, amg_setup.cpp): aggregation, tentative
 * prolongators from the six rigid-body modes of the reference configuration,
 * and the block patterns of P, A P and P^T A P on every level.  Numeric part
 * (device, once per tangent, amg.cu): block-diagonal inverses, spectral
 * radius of D^-1 A by power iteration, the smoothed prolongator
 * P = (I - omega D^-1 A) P_tent with omega = 4 / (3 lambda_max), the Galerkin
 * products and the dense inverse of the coarsest operator.  The V-cycle runs
 * in FP32 with Chebyshev(2) / block-Jacobi smoothing.
 *
 * Rows that the tangent holds as identity (clamped nodes and ghost nodes) take
 * no part in the aggregation: their prolongator rows are zero and the smoother
 * alone acts on them.
 */
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace biofem {

constexpr int kAmgCoarseBs = 6;      /* rigid-body modes per aggregate */
constexpr int kAmgMaxDense = 192;    /* coarsest operator solved densely up to this many unknowns */
constexpr int kAmgMaxLevels = 10;

struct AmgLevelHost {
  int n = 0, bs = 0, na = 0;                 /* nodes, block size, aggregates (0 on the coarsest) */
  std::vector<int> rowptr, colind, diag;     /* operator pattern (block CSR) and the diagonal block per row */
  std::vector<int> agg;                      /* node -> aggregate, -1 when excluded */
  std::vector<float> Q;                      /* n * bs * 6 tentative prolongator rows */
  std::vector<unsigned char> dead;           /* na * 6: coarse unknowns with no tentative column */
  std::vector<int> prow, pcol, pblkrow;      /* P pattern (fine row -> aggregates) and block -> row */
  std::vector<int> rrow, rcol, rmap;         /* P^T pattern: aggregate -> fine rows, and the P block of each */
  std::vector<int> trow, tcol, tblkrow;      /* T = A P pattern */
  std::vector<int> crow, ccol, cblkrow;      /* next level's operator pattern */
};

/* Build the symbolic hierarchy.  rowptr/colind: the nt-row block pattern of
   the tangent; rowkind: 0 for a free row, nonzero for an identity row; X:
   3*nt reference positions; tri: ntri real triangles (level-0 aggregation
   graph).  Returns the number of levels (>= 1). */
int amg_symbolic(int nt, const std::vector<int> &rowptr, const std::vector<int> &colind,
                 const std::vector<unsigned char> &rowkind, const std::vector<double> &X, const int *tri, int ntri,
                 std::vector<AmgLevelHost> &levels);

struct AmgHier;

/* Symbolic setup and device allocations (stream-ordered on st). */
AmgHier *amg_create(int nt, const std::vector<int> &rowptr, const std::vector<int> &colind,
                    const std::vector<unsigned char> &rowkind, const std::vector<double> &X, const int *tri, int ntri,
                    const int *d_rowptr, const int *d_colind, bool k_is_f32, cudaStream_t st, int *rc);
void amg_destroy(AmgHier *h);
/* Numeric setup from the current tangent values (FP32 blocks, or FP64 blocks
   converted into a copy when the hierarchy was created with k_is_f32 false). */
int amg_numeric(AmgHier *h, const void *K, bool k_is_f32, cudaStream_t st);
/* z = M^-1 v for FP64 vectors of 3*nt entries; kernels skip their work while
   *done is nonzero (done may be null). */
void amg_apply(AmgHier *h, const double *v, double *z, const int *done, cudaStream_t st);
int amg_levels(const AmgHier *h);
long long amg_device_bytes(const AmgHier *h);

}  // namespace biofem

// ref_ops.cpp -- C entry points to single operators of the reference's own 2D
// sources compiled for the CPU (TEST INFRASTRUCTURE ONLY: the checker's
// checker, never part of the product).
//
// oracle/build_ref.py links this file against libref_deformation_2D_frame.so
// (the reference's CUDA/2D_frame sources and the CPU emulation of
// oracle/ref_shim), so each entry point below runs the reference's own
// kernels.  Only the reference functions' names and signatures are declared
// here; all "device" pointers are host memory under the emulation.  Layouts
// are the reference's: nodes and nodal vectors N x 2 column-major, index
// matrices entity-index fastest, dense matrices N x N column-major.
//
// tests/golden/make_layered_pin.py uses them to pin the layered (isotropic)
// operators of oracle/oracle.c where they coincide with the frame model's:
// 2D frame elasticity with mu_tan = mu_tsv = mu_ang = 2 mu on an orthonormal
// frame is isotropic elasticity with lambda = 0; anisotropic diffusion with
// spdTan = spdTsv = D is isotropic diffusion; the mass matrix, the yank load
// (-f I with the element mean of a given nodal activity) and the reaction
// load (consistent mass times a given activity) are the same operators.
#include <cstdlib>
#include <cstring>
#include <vector>

// the reference's functions (CUDA/2D_frame/*.cu), resolved in libref_deformation_2D_frame.so
void vertexToEdge(double *, double *, int *, int, int);                                          // vertexToEdge.cu:29
void vertexToBottom(double *, double *, int *, int, int);                                        // vertexToBottom.cu:23
void computeFrame(double *, double *, double *, int *, int *, int, int);                         // computeFrame.cu:70
void applyFrameElasticOperator(double *, double *, double *, double *, double *, double *, double *, double *,
                               int *, int *, int, int);                                          // applyFrameElasticOperator.cu:113
void assembleFemMatrix(double *, double *, double *, double *, double *, double, double, double *, double *,
                       int *, int *, int, int, int);                                             // assembleFemMatrix.cu:94
void assembleFemVector(double *, double *, double *, double *, int *, int *, int, int);          // assembleFemVector.cu:56
void computeExternalYank(double *, double *, double *, double *, double *, double *, int *, int *, int *, int *,
                         int, int, int);                                                        // computeExternalYank.cu:124
void applyPenaltyOperator(double *, double *, double *, double *, int *, int *, int, int, int);  // applyPenaltyOperator.cu:65

namespace {
constexpr int D = 2, V = 3;

template <typename T> T *mut(const T *p) { return const_cast<T *>(p); }

std::vector<double> edges(int N, int E, const double *lmk, const int *elmVtx)
{
	std::vector<double> e((size_t) E * D * (V - 1));
	vertexToEdge(e.data(), mut(lmk), mut(elmVtx), N, E);
	return e;
}
}  // namespace

extern "C" {

// y = E v: frame elasticity with modVec = (muTan, muTsv, muAng) on the frame of the current shape
int refop_elastic(int N, int E, const double *lmk, const int *elmVtx, const int *vtxElm, const int *tanVtx,
                  const int *tsvVtx, const double *modVec, const double *v, double *y)
{
	std::vector<double> edg = edges(N, E, lmk, elmVtx);
	std::vector<double> tan((size_t) E * D), tsv((size_t) E * D);
	computeFrame(tan.data(), tsv.data(), mut(lmk), mut(tanVtx), mut(tsvVtx), N, E);
	std::vector<double> epv((size_t) E * D * D), elYElm((size_t) E * V * D);
	applyFrameElasticOperator(y, edg.data(), tan.data(), tsv.data(), mut(modVec), mut(v), epv.data(), elYElm.data(),
	                          mut(elmVtx), mut(vtxElm), N, E);
	return 0;
}

// dense mass (ppd) and diffusion (ggd) matrices, N x N column-major
int refop_fem_matrix(int N, int E, int Z, const double *lmk, const int *elmVtx, const int *tanVtx,
                     const int *tsvVtx, const int *femVtx, const int *femIfo, double spdTan, double spdTsv,
                     double *ppd, double *ggd)
{
	std::vector<double> edg = edges(N, E, lmk, elmVtx);
	std::vector<double> tan((size_t) E * D), tsv((size_t) E * D);
	computeFrame(tan.data(), tsv.data(), mut(lmk), mut(tanVtx), mut(tsvVtx), N, E);
	std::vector<double> ppdElm((size_t) E), ggdElm((size_t) E * 6);
	assembleFemMatrix(ppd, ggd, edg.data(), tan.data(), tsv.data(), spdTan, spdTsv, ppdElm.data(), ggdElm.data(),
	                  mut(femVtx), mut(femIfo), N, Z, E);
	return 0;
}

// y_i = sum_e int f phi_i (consistent mass), f a nodal activity
int refop_fem_vector(int N, int E, const double *lmk, const int *elmVtx, const int *vtxElm, const double *act,
                     double *y)
{
	std::vector<double> edg = edges(N, E, lmk, elmVtx);
	std::vector<double> rpdElm((size_t) E * V);
	assembleFemVector(y, edg.data(), mut(act), rpdElm.data(), mut(elmVtx), mut(vtxElm), N, E);
	return 0;
}

// y = yank load of the nodal activity f (element mean of f times -I, against the basis gradients)
int refop_yank(int N, int E, int bdrNum, const double *lmk, const int *elmVtx, const int *vtxElm, const int *bdrVtx,
               const int *vtxBdr, const double *act, double *y)
{
	std::vector<double> edg = edges(N, E, lmk, elmVtx);
	std::vector<double> exYElm((size_t) E * V * D), exYBdr((size_t) (bdrNum > 0 ? bdrNum : 1) * 2 * D);
	computeExternalYank(y, mut(lmk), edg.data(), mut(act), exYElm.data(), exYBdr.data(), mut(elmVtx), mut(vtxElm),
	                    mut(bdrVtx), mut(vtxBdr), N, E, bdrNum);
	return 0;
}

// y = P v (bottom penalty, lumped on the bottom segments); y has N rows, the bottom nodes' rows are written
int refop_penalty(int N, int Bt, int Nb, const double *lmk, const int *btmVtx, const int *vtxBtm, const double *v,
                  double *y)
{
	std::vector<double> btm((size_t) Bt * D * D), pnlBtm((size_t) Bt * 2 * D);
	vertexToBottom(btm.data(), mut(lmk), mut(btmVtx), N, Bt);
	applyPenaltyOperator(y, btm.data(), mut(v), pnlBtm.data(), mut(btmVtx), mut(vtxBtm), N, Bt, Nb);
	return 0;
}

}  // extern "C"

// MEX gateway deformation_2D_isotropic / deformation_3D_isotropic: the layered (isotropic) model for the
// branch that CUDA/deformation.m:12-13,22-24 parses and leaves empty.  Right-hand sides are those of
// deformation_{2D,3D}_frame (CUDA/2D_frame/deformation.cu:24-50) with three changes:
//   prhs[13]  elmObj.elmLyrVec            gpuArray int32, E      (0-based material layer of each element)
//   prhs[18]  d_modMat                    gpuArray, lyrNum x 2   (reshape(h_modVec, 2, [])': lambda, mu)
//   prhs[19]  per-layer diffusivities     host, lyrNum           (the wrapper's spdTanVal(:))
// so the frame's ldmWgt..knlEps move to prhs[14..17] and spdTsvVal is dropped (27 arguments).  prhs[5..6]
// (tanVtxMat/nmlVtxMat, tsvVtxMat) are not used by this model and may be empty.  Outputs as the frame
// gateway: lmkStk (N*dim) x timeNum, tauMat N x timeNum, objVec 1 x nObj (host).
//
// Build (MATLAB):
//   mex -R2018a -DSA_DIM=2 sa_mex_deformation_isotropic.cpp -I<repo>/include \
//       -L<repo>/shape_atrophy_gb300/_build -lshape_atrophy_gb300 -output deformation_2D_isotropic
#include "mex.h"
#include "gpu/mxGPUArray.h"
#include "shape_atrophy_gb300.h"

#ifndef SA_DIM
#error "define SA_DIM=2 or SA_DIM=3"
#endif

static sa_context *g_ctx = nullptr;

static void release_context()
{
	sa_destroy(g_ctx);
	g_ctx = nullptr;
}

// device (or host) data and the two leading dimensions of a gpuArray argument
template <typename T>
static const T *gpu_arg(const mxArray *a, const mxGPUArray **keep, int *rows, int *cols)
{
	*keep = mxGPUCreateFromMxArray(a);
	const mwSize *d = mxGPUGetDimensions(*keep);
	if (rows) *rows = (int) d[0];
	if (cols) *cols = (int) d[1];
	mxFree((void *) d);
	return (const T *) mxGPUGetDataReadOnly(*keep);
}

void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[])
{
	(void) nlhs;
	if (nrhs != 27) mexErrMsgIdAndTxt("sa:deformation", "27 input arguments expected, got %d", nrhs);
	mxInitGPU();
	if (!g_ctx) {
		if (sa_create(&g_ctx, 0) != SA_OK) mexErrMsgIdAndTxt("sa:deformation", "no usable GPU");
		mexAtExit(release_context);
	}
	const mxGPUArray *keep[13];
	int N, E, dummy, vtxElmCols, frmRows, tsvRows, bdrNum, vtxBdrCols, btmNum, btmLmkNum, vtxBtmCols, nzr,
	    femIfoCols, lyrNum, lyrCols;
	const double *lmk = gpu_arg<double>(prhs[2], &keep[0], &N, &dummy);
	const int *elm = gpu_arg<int>(prhs[3], &keep[1], &E, &dummy);
	const int *vtxElm = gpu_arg<int>(prhs[4], &keep[2], &dummy, &vtxElmCols);
	const int *frm = gpu_arg<int>(prhs[5], &keep[3], &frmRows, nullptr);
	const int *tsv = gpu_arg<int>(prhs[6], &keep[4], &tsvRows, nullptr);
	const int *bdr = gpu_arg<int>(prhs[7], &keep[5], &bdrNum, &dummy);
	const int *vtxBdr = gpu_arg<int>(prhs[8], &keep[6], &dummy, &vtxBdrCols);
	const int *btm = gpu_arg<int>(prhs[9], &keep[7], &btmNum, &dummy);
	const int *vtxBtm = gpu_arg<int>(prhs[10], &keep[8], &btmLmkNum, &vtxBtmCols);
	const int *femVtx = gpu_arg<int>(prhs[11], &keep[9], &nzr, &dummy);
	const int *femIfo = gpu_arg<int>(prhs[12], &keep[10], &dummy, &femIfoCols);
	const int *elmLyr = gpu_arg<int>(prhs[13], &keep[11], nullptr, nullptr);
	const double *modMat = gpu_arg<double>(prhs[18], &keep[12], &lyrNum, &lyrCols);
	const int nVar = (int) mxGetM(prhs[0]), nObj = (int) mxGetN(prhs[0]);
	const int timeNum = (int) mxGetScalar(prhs[24]);
	if (lyrCols != 2 || (int) mxGetNumberOfElements(prhs[19]) != lyrNum) {
		for (const mxGPUArray *a : keep) mxGPUDestroyGPUArray(a);
		mexErrMsgIdAndTxt("sa:deformation", "modMat must be lyrNum x 2 and the diffusivities lyrNum values");
	}
	plhs[0] = mxCreateDoubleMatrix((mwSize) N * SA_DIM, (mwSize) timeNum, mxREAL);
	plhs[1] = mxCreateDoubleMatrix((mwSize) N, (mwSize) timeNum, mxREAL);
	plhs[2] = mxCreateDoubleMatrix(1, (mwSize) nObj, mxREAL);
	int rc = sa_deformation_isotropic(g_ctx, SA_DIM,
		mxGetDoubles(prhs[0]), nVar, nObj, mxGetDoubles(prhs[1]), (int) mxGetNumberOfElements(prhs[1]),
		lmk, N, elm, E, vtxElm, vtxElmCols, frmRows == E ? frm : nullptr, tsvRows == E ? tsv : nullptr,
		bdr, bdrNum, vtxBdr, vtxBdrCols, btm, btmNum, vtxBtm, btmLmkNum, vtxBtmCols, femVtx, nzr, femIfo,
		femIfoCols, elmLyr,
		mxGetScalar(prhs[14]), (int) mxGetScalar(prhs[15]), mxGetScalar(prhs[16]), mxGetScalar(prhs[17]),
		modMat, lyrNum, mxGetDoubles(prhs[19]),
		mxGetDoubles(prhs[20]), mxGetDoubles(prhs[21]), mxGetScalar(prhs[22]), mxGetScalar(prhs[23]), timeNum,
		(int) mxGetScalar(prhs[25]), mxGetScalar(prhs[26]),
		mxGetDoubles(plhs[0]), mxGetDoubles(plhs[1]), mxGetDoubles(plhs[2]));
	for (const mxGPUArray *a : keep) mxGPUDestroyGPUArray(a);
	if (rc != SA_OK) mexErrMsgIdAndTxt("sa:deformation", "%s", sa_error_message(g_ctx));
}

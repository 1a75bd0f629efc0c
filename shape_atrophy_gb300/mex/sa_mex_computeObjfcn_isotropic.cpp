// MEX gateway computeObjfcn_2D_isotropic / computeObjfcn_3D_isotropic: the layered (isotropic) model for
// the branch that CUDA/computeObjfcn.m:12-13,22-24 parses and leaves empty.  Right-hand sides are those of
// computeObjfcn_{2D,3D}_frame (CUDA/2D_frame/computeObjfcn.cu:25-59) with the changes of the isotropic
// deformation gateway: elmObj.elmLyrVec (gpuArray int32, E) is prhs[13], so the varifold arguments move to
// prhs[14..21] and ldmWgt..knlEps to prhs[22..25]; d_modMat (gpuArray lyrNum x 2, reshape(h_modVec, 2,
// [])') is prhs[26]; the per-layer diffusivities (host, lyrNum) are prhs[27]; spdTsvVal is dropped (35
// arguments).  Output objVec 1 x nObj (DBL_MAX for a column whose velocity solve failed).
//
// Build (MATLAB):
//   mex -R2018a -DSA_DIM=2 sa_mex_computeObjfcn_isotropic.cpp -I<repo>/include \
//       -L<repo>/shape_atrophy_gb300/_build -lshape_atrophy_gb300 -output computeObjfcn_2D_isotropic
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
	if (nrhs != 35) mexErrMsgIdAndTxt("sa:computeObjfcn", "35 input arguments expected, got %d", nrhs);
	mxInitGPU();
	if (!g_ctx) {
		if (sa_create(&g_ctx, 0) != SA_OK) mexErrMsgIdAndTxt("sa:computeObjfcn", "no usable GPU");
		mexAtExit(release_context);
	}
	const mxGPUArray *keep[17];
	int N, E, dummy, vtxElmCols, frmRows, tsvRows, bdrNum, vtxBdrCols, btmNum, btmLmkNum, vtxBtmCols, nzr,
	    femIfoCols, Vd, Vt, lyrNum, lyrCols;
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
	const int *vfdVtx = gpu_arg<int>(prhs[14], &keep[12], &Vd, &dummy);
	const double *cen = gpu_arg<double>(prhs[15], &keep[13], nullptr, nullptr);
	const double *dir = gpu_arg<double>(prhs[16], &keep[14], nullptr, nullptr);
	const double *vol = gpu_arg<double>(prhs[17], &keep[15], &Vt, &dummy);
	const double *modMat = gpu_arg<double>(prhs[26], &keep[16], &lyrNum, &lyrCols);
	const int nVar = (int) mxGetM(prhs[0]), nObj = (int) mxGetN(prhs[0]);
	if (lyrCols != 2 || (int) mxGetNumberOfElements(prhs[27]) != lyrNum) {
		for (const mxGPUArray *a : keep) mxGPUDestroyGPUArray(a);
		mexErrMsgIdAndTxt("sa:computeObjfcn", "modMat must be lyrNum x 2 and the diffusivities lyrNum values");
	}
	plhs[0] = mxCreateDoubleMatrix(1, (mwSize) nObj, mxREAL);
	int rc = sa_computeObjfcn_isotropic(g_ctx, SA_DIM,
		mxGetDoubles(prhs[0]), nVar, nObj, mxGetDoubles(prhs[1]), (int) mxGetNumberOfElements(prhs[1]),
		lmk, N, elm, E, vtxElm, vtxElmCols, frmRows == E ? frm : nullptr, tsvRows == E ? tsv : nullptr,
		bdr, bdrNum, vtxBdr, vtxBdrCols, btm, btmNum, vtxBtm, btmLmkNum, vtxBtmCols, femVtx, nzr, femIfo,
		femIfoCols, elmLyr, vfdVtx, Vd, cen, dir, vol, Vt,
		mxGetScalar(prhs[18]), mxGetScalar(prhs[19]), mxGetScalar(prhs[20]), mxGetScalar(prhs[21]),
		mxGetScalar(prhs[22]), (int) mxGetScalar(prhs[23]), mxGetScalar(prhs[24]), mxGetScalar(prhs[25]),
		modMat, lyrNum, mxGetDoubles(prhs[27]),
		mxGetDoubles(prhs[28]), mxGetDoubles(prhs[29]), mxGetScalar(prhs[30]), mxGetScalar(prhs[31]),
		(int) mxGetScalar(prhs[32]), (int) mxGetScalar(prhs[33]), mxGetScalar(prhs[34]),
		mxGetDoubles(plhs[0]));
	for (const mxGPUArray *a : keep) mxGPUDestroyGPUArray(a);
	if (rc != SA_OK) mexErrMsgIdAndTxt("sa:computeObjfcn", "%s", sa_error_message(g_ctx));
}

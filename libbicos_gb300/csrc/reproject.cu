// Point-cloud reprojection of a disparity map (the step after the match in
// libBICOS's bicos-cli, src/cli.cpp:228-250: cv::reprojectImageTo3D(disp,
// points, Q, false, CV_32F)).  Each pixel (x, y) with disparity d maps to
// the homogeneous point  [X Y Z W]^T = Q [x y d 1]^T  and is written as the
// three floats (X/W, Y/W, Z/W); W = 0 gives (0, 0, 0), as in OpenCV.  Every
// pixel is reprojected, invalid disparities included (INT16_MIN as a value,
// NaN propagating); the point-cloud writer skips them.
//
// One thread per pixel, FP32 arithmetic (X, Y, Z, W as fused sums of the
// Q terms, reproject_store in kernels.cuh): HBM-bound, 2 or 4 bytes in and
// 12 bytes out per pixel.  bicos_match_points_v1 writes the same points
// from the agreement kernels' epilogue instead (no second pass).
#include "kernels.cuh"

namespace bicos_gb300 {
namespace {

template<typename D>
__global__ void __launch_bounds__(256) k_reproject(const __grid_constant__ ReprojectParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= p.cols)
        return;
    const D* drow = reinterpret_cast<const D*>(reinterpret_cast<const char*>(p.disp) + (long long)y * p.disp_pitch);
    reproject_store(p.q, reinterpret_cast<float*>(reinterpret_cast<char*>(p.pts) + (long long)y * p.pts_pitch), x, y,
                    (float)drow[x]);
}

}  // namespace

cudaError_t launch_reproject(const ReprojectParams& p, bool float_disp, cudaStream_t st) {
    const dim3 grid((p.cols + 255) / 256, p.rows);
    if (float_disp)
        k_reproject<float><<<grid, 256, 0, st>>>(p);
    else
        k_reproject<int16_t><<<grid, 256, 0, st>>>(p);
    return cudaGetLastError();
}

}  // namespace bicos_gb300

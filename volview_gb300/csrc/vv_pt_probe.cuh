// vv_pt_probe.cuh — the single-path probe: pt.comp's per-pixel result for a
// list of pixels, one thread per pixel, at accumulation count a.u.path[0].
// Included inside the format namespace of vv_pt.cu (the product's samplers)
// and of vv_pt_exact.cu (the parity build, compiled with --fmad=false).
#pragma once

__global__ void k_pt_pixels(const __grid_constant__ PtArgs A, const int* pix, float* out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t px = (uint32_t)pix[2 * i], py = (uint32_t)pix[2 * i + 1];
    Consts C = make_consts(A);
    Path P;
    PixelSums S = {mk(0.0f), 0.0f, make_float4(0, 0, 0, 0), make_float4(0, 0, 0, 0)};
    P.rng.s = seed_of(px, py, A.u.path[0]);
    P.rng.pcg();
    for (uint32_t k = 0; k < A.u.path[2]; k++) {
        start_path(A, C, P, px, py);
        while (bounce_step(A, C, P, S)) {
        }
        finish_path(P, S);
    }
    float* o = out + 12 * i;
    o[0] = S.sum.x; o[1] = S.sum.y; o[2] = S.sum.z; o[3] = S.background;
    o[4] = S.albedo.x; o[5] = S.albedo.y; o[6] = S.albedo.z; o[7] = S.albedo.w;
    o[8] = S.normal.x; o[9] = S.normal.y; o[10] = S.normal.z; o[11] = S.normal.w;
}
cudaError_t launch_pt_pixels(const PtArgs& a, const int* px, float* out, int n, cudaStream_t s) {
    k_pt_pixels<<<(n + 63) / 64, 64, 0, s>>>(a, px, out, n);
    return cudaGetLastError();
}

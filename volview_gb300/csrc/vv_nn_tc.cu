// vv_nn_tc.cu — the learned denoiser's 3x3 convolution on the fifth-generation
// tensor cores: tcgen05.mma (kind::f16, FP16 operands from shared memory, FP32
// accumulators in tensor memory) fed by TMA (cp.async.bulk.tensor).
//
// Implicit GEMM over 128-pixel segments of image rows (widths that are
// multiples of 128): M = the segment's 128 output pixels, N = the output
// channels padded to a multiple of 16, K = 9 taps x the input channels.
// Operands are K-major in the canonical no-swizzle layout: 8-row x 16-byte
// core matrices, the 8-row groups of one 16-byte K slice 128 bytes apart (the
// stride byte offset), consecutive K slices LBO bytes apart.
//
// A CTA keeps all nine taps' weights in shared memory and walks down a run
// of rows of one column of segments (the same 128 pixels of consecutive
// rows). Its input rows, each with its one-pixel halo (130 pixels), sit in a
// ring of four row slots: a segment uses three (rows y-1, y, y+1) and the
// fourth takes the next row, so every input row is copied once per run. TMA
// copies a row as boxes of 8 channels x 130 pixels, one per 16-byte channel
// slice, zero-filled outside the image (same padding); such a box is one K
// slice of the layout above. Tap (dy, dx)'s A operand is row y+dy-1's slices
// starting dx pixels in: the descriptor's start address moves by 16 bytes per
// pixel. Roles:
//   warp 4 (one lane): waits for a segment's three rows, issues its
//     9 x cin / 16 MMAs into one of two TMEM accumulators, commits them to an
//     mbarrier, and copies the next row into the slot the previous segment
//     has finished with;
//   warps 0-3: read the finished accumulator (warp w owns TMEM lanes
//     32w..32w+31, one output pixel per lane), release it, add the bias,
//     apply the ReLU and store FP16.
// So a segment's copies, the next segment's MMAs and the previous segment's
// epilogue overlap. Every wait on an mbarrier is bounded: past the limit the
// thread records the failure in a device status word (vv_nn_tc_status) and
// goes on, and the CTA still frees its tensor memory.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/volpt_nn.h"

namespace vv {
namespace nn {

__device__ int g_tc_status;  // 0, or 1 after a bounded wait gave up

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor (tcgen05): start address, leading (K) and
// stride (M/N) byte offsets, each >> 4; bits 46-48 = 0b001; base offset 0,
// relative leading offset, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), FP16 A
// and B (bits 7-9, 10-12 = 0), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0));
}

// Waits until the mbarrier's phase of parity `parity` has completed; false
// when the bounded wait gave up (the status word is set).
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity) {
    for (int it = 0; it < (1 << 22); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicExch(&g_tc_status, 1);
    return false;
}

constexpr int TC_M = 128;                     // output pixels per segment (TMEM lanes)
constexpr int HALO = TC_M + 2;                // input pixels per row slice
constexpr int SLICE = HALO * 16;              // bytes of one 8-channel slice of a row (one TMA box)
constexpr int SLICE_STRIDE = 136 * 16;        // its stride in shared memory, a multiple of the 128 bytes TMA
                                              // destinations need: the A operand's LBO
constexpr int EPI_THREADS = 128;              // warps 0-3
constexpr int TC_THREADS = EPI_THREADS + 32;  // + warp 4, the issuing warp

__host__ __device__ constexpr uint32_t tmem_cols(int np) {
    return 2 * np <= 32 ? 32 : 2 * np <= 64 ? 64 : 2 * np <= 128 ? 128 : 2 * np <= 256 ? 256 : 512;
}
// Row slots of the ring: four (a segment reads three while the next row
// loads), or three where that fits twice as many CTAs in an SM's shared memory
// (the next row then loads once the segment's MMAs are done with its slot).
constexpr int RING = 4;
// Weights, the ring of row slots, and slack to align the ring to 1024 bytes.
static size_t tc_smem(int np, int cin, int ring = RING) {
    return 9 * (size_t)np * 2 * cin + ring * (size_t)(cin / 8) * SLICE_STRIDE + 1024;
}

template <int NP, int RING>
__global__ void __launch_bounds__(TC_THREADS) k_conv3x3_tc(const __grid_constant__ CUtensorMap rows, int n, int h,
                                                           int w, int cin, const __half* __restrict__ wt,
                                                           const float* __restrict__ bias, int cout, int relu,
                                                           __half* __restrict__ y, int run_rows) {
    constexpr uint32_t COLS = tmem_cols(NP);
    constexpr uint32_t IDESC = instr_desc(TC_M, NP);
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bars[RING + 4];  // full[RING] (TMA), mma[2] (tcgen05.commit), free[2]
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int chunks = cin >> 3;
    const int per_row = w / TC_M;
    // This CTA's run: column (image, segment) blockIdx.x % columns, rows
    // [y0, y1) of it.
    const int columns = n * per_row;
    const int column = (int)(blockIdx.x % columns), run = (int)(blockIdx.x / columns);
    const int img = column / per_row, x0 = (column - img * per_row) * TC_M;
    const int y0 = run * run_rows, y1 = min(h, y0 + run_rows);
    const int ntiles = y1 > y0 ? y1 - y0 : 0;
    const uint32_t wbase = smem_u32(smem);
    const uint32_t w_tap = NP * 2 * cin;                        // one tap's weights
    const uint32_t hbase = (wbase + 9 * w_tap + 1023u) & ~1023u;  // the ring of row slots
    const uint32_t seg = chunks * SLICE_STRIDE;                 // one row slot
    const uint32_t full0 = smem_u32(&bars[0]), mma0 = smem_u32(&bars[RING]), free0 = smem_u32(&bars[RING + 2]);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int k = 0; k < RING; k++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8 * k));
        for (int k = 0; k < 2; k++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mma0 + 8 * k));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(free0 + 8 * k), "r"(EPI_THREADS));
        }
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    // Every tap's weights, rows padded to NP with zeros: 16-byte copies by all threads.
    {
        const int per_tap = NP * chunks;
        for (int j = tid; j < 9 * per_tap; j += TC_THREADS) {
            const int tap = j / per_tap, rem = j - tap * per_tap;
            const int r = rem % NP, c = rem / NP;
            const bool ok = r < cout;
            const __half* src = ok ? wt + ((long)r * 9 + tap) * cin + c * 8 : wt;
            cp_async16(wbase + tap * w_tap + c * (NP * 16) + r * 16, src, ok);
        }
        asm volatile("cp.async.commit_group;");
        asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t tmem = tmem_slot;

    if (warp == 4) {
        if (lane == 0 && ntiles > 0) {
            const uint32_t bytes = chunks * SLICE;
            // Relative row q of the run is image row y0 - 1 + q, in slot q % RING;
            // its copy is that slot's (q / RING)-th.
            auto load_row = [&](int q) {
                const uint32_t bar = full0 + 8 * (q % RING);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
                for (int c = 0; c < chunks; c++) {
                    const uint32_t dst = hbase + (q % RING) * seg + c * SLICE_STRIDE;
                    asm volatile(
                        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
                        "l"((uint64_t)&rows), "r"(c * 8), "r"(x0 - 1), "r"(y0 - 1 + q), "r"(img), "r"(bar)
                        : "memory");
                }
            };
            load_row(0);
            load_row(1);
            load_row(2);
            for (int i = 0; i < ntiles; i++) {
                const int b = i & 1;
                for (int q = i; q < i + 3; q++) bar_wait(full0 + 8 * (q % RING), (q / RING) & 1);  // rows y-1, y, y+1
                if (i >= 2) bar_wait(free0 + 8 * b, ((i >> 1) - 1) & 1);  // accumulator b read out
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + b * NP;
                for (int tap = 0; tap < 9; tap++) {
                    const uint32_t a0 = hbase + ((i + tap / 3) % RING) * seg + (tap % 3) * 16;
                    const uint32_t b0 = wbase + tap * w_tap;
                    for (int k = 0; k < cin / 16; k++) {
                        const uint64_t da = smem_desc(a0 + k * 2 * SLICE_STRIDE, SLICE_STRIDE, 128);
                        const uint64_t db = smem_desc(b0 + k * 2 * NP * 16, NP * 16, 128);
                        const uint32_t accumulate = (tap > 0 || k > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(acc),
                            "l"(da), "l"(db), "r"(IDESC), "r"(accumulate));
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mma0 + 8 * b)
                             : "memory");
                if (i + 1 < ntiles) {
                    // The next segment's new row goes into the slot of row
                    // i + 3 - RING, which segment i + 3 - RING's MMAs were the
                    // last to read (the previous segment's with four slots, this
                    // one's with three).
                    const int last = i + 3 - RING;
                    if (last >= 0) bar_wait(mma0 + 8 * (last & 1), (last >> 1) & 1);
                    load_row(i + 3);
                }
            }
        }
        __syncwarp();
    } else {
        // Epilogue: warps 0-3, one output pixel per thread.
        for (int i = 0; i < ntiles; i++) {
            const int b = i & 1;
            const bool ok = bar_wait(mma0 + 8 * b, (i >> 1) & 1);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            uint32_t packed[NP / 2];
            const uint32_t row_addr = tmem + b * NP + ((uint32_t)(warp * 32) << 16);
#pragma unroll
            for (int c0 = 0; c0 < NP; c0 += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                    "[%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                      "=r"(r[15])
                    : "r"(row_addr + c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    float v0 = __uint_as_float(r[2 * j]), v1 = __uint_as_float(r[2 * j + 1]);
                    const int co = c0 + 2 * j;
                    if (bias && co < cout) v0 += __ldg(bias + co);
                    if (bias && co + 1 < cout) v1 += __ldg(bias + co + 1);
                    if (relu) {
                        v0 = fmaxf(v0, 0.0f);
                        v1 = fmaxf(v1, 0.0f);
                    }
                    packed[c0 / 2 + j] = (uint32_t)__half_as_ushort(__float2half_rn(v0)) |
                                         ((uint32_t)__half_as_ushort(__float2half_rn(v1)) << 16);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(free0 + 8 * b) : "memory");
            if (ok) {
                const long p = ((long)img * h + y0 + i) * w + x0 + tid;
                __half* dst = y + p * cout;
#pragma unroll
                for (int c0 = 0; c0 < NP; c0 += 8)
                    if (c0 < cout)
                        *(uint4*)(dst + c0) = make_uint4(packed[c0 / 2], packed[c0 / 2 + 1], packed[c0 / 2 + 2],
                                                         packed[c0 / 2 + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(COLS));
}

// The input tensor (n, h, w, cin) FP16 as a 4-D TMA map, innermost first:
// channels, pixels, rows, images; boxes of 8 channels x 130 pixels x 1 x 1.
static bool encode_rows_map(CUtensorMap* map, const void* x, int n, int h, int w, int cin) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return false;
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    const cuuint64_t dims[4] = {(cuuint64_t)cin, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)n};
    const cuuint64_t strides[3] = {(cuuint64_t)cin * 2, (cuuint64_t)w * cin * 2, (cuuint64_t)h * w * cin * 2};
    const cuuint32_t box[4] = {8, HALO, 1, 1};
    const cuuint32_t elem[4] = {1, 1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 4, const_cast<void*>(x), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Resident CTAs per SM for `smem` bytes of dynamic shared memory: by shared
// memory (with 1 KB per CTA the system reserves and the static barriers), by
// threads, and by TMEM (at most 512 columns per SM between them, so that no
// allocation waits).
static int resident_ctas(size_t smem, int np, int sm_smem) {
    int per_sm = sm_smem / (int)(smem + 2048);
    per_sm = per_sm < 2048 / TC_THREADS ? per_sm : 2048 / TC_THREADS;
    per_sm = per_sm < (int)(512 / tmem_cols(np)) ? per_sm : (int)(512 / tmem_cols(np));
    return per_sm < 1 ? 1 : per_sm;
}

template <int NP, int RING>
static cudaError_t launch_tc(const CUtensorMap& map, int n, int h, int w, int cin, const __half* wt, const float* bias,
                             int cout, int relu, __half* y, cudaStream_t s, int sms, int per_sm) {
    const size_t smem = tc_smem(NP, cin, RING);
    static bool configured = false;
    if (!configured) {
        cudaError_t e =
            cudaFuncSetAttribute(k_conv3x3_tc<NP, RING>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    // Runs of rows: every resident CTA takes one, the runs of a column of
    // segments as long as the CTAs per column allow.
    const long columns = (long)n * (w / TC_M);
    const long slots = (long)sms * per_sm;
    const long per_column = std::max(1L, slots / columns);
    const int run_rows = (int)((h + per_column - 1) / per_column);
    const long grid = columns * ((h + run_rows - 1) / run_rows);
    k_conv3x3_tc<NP, RING><<<(unsigned)grid, TC_THREADS, smem, s>>>(map, n, h, w, cin, wt, bias, cout, relu, y,
                                                                    run_rows);
    return cudaGetLastError();
}

// Four row slots, or three where that fits more CTAs per SM (the U-Net's
// full-resolution decoder, 80 -> 32 channels: one CTA per SM with four slots,
// two with three).
template <int NP>
static cudaError_t launch_tc_ring(const CUtensorMap& map, int n, int h, int w, int cin, const __half* wt,
                                  const float* bias, int cout, int relu, __half* y, cudaStream_t s) {
    int dev = 0, sms = 0, sm_smem = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e != cudaSuccess) return e;
    const int four = resident_ctas(tc_smem(NP, cin, 4), NP, sm_smem);
    const int three = resident_ctas(tc_smem(NP, cin, 3), NP, sm_smem);
    if (four == 1 && three > 1)
        return launch_tc<NP, 3>(map, n, h, w, cin, wt, bias, cout, relu, y, s, sms, three);
    return launch_tc<NP, 4>(map, n, h, w, cin, wt, bias, cout, relu, y, s, sms, four);
}

// The tensor-core convolution when the shape suits it (widths that are
// multiples of 128, cout <= 96 and the weights and two segments' rows within
// 220 KB of shared memory); returns false to leave the shape to the mma.sync
// convolution. *err receives the launch's error.
bool conv3x3_tc(const __half* x, int n, int h, int w, int cin, const __half* wt, const float* bias, int cout,
                int relu, __half* y, cudaStream_t s, cudaError_t* err) {
    const int np = (cout + 15) / 16 * 16;
    if (w % TC_M || np > 96 || tc_smem(np, cin) > 220 * 1024) return false;
    if (((uintptr_t)x | (uintptr_t)wt | (uintptr_t)y) % 16) return false;
    CUtensorMap map;
    if (!encode_rows_map(&map, x, n, h, w, cin)) return false;
    switch (np) {
        case 16: *err = launch_tc_ring<16>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        case 32: *err = launch_tc_ring<32>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        case 48: *err = launch_tc_ring<48>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        case 64: *err = launch_tc_ring<64>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        case 80: *err = launch_tc_ring<80>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        case 96: *err = launch_tc_ring<96>(map, n, h, w, cin, wt, bias, cout, relu, y, s); break;
        default: return false;
    }
    return true;
}

}  // namespace nn
}  // namespace vv

using namespace vv::nn;

extern "C" vv_status vv_nn_conv3x3_tc(const void* x, int n, int h, int w, int cin, const void* weights,
                                      const float* bias, int cout, int relu, void* y, void* stream) {
    if (!x || !weights || !y || n <= 0 || h <= 0 || w <= 0 || w % 16 || cin <= 0 || cin % 16 || cout <= 0 ||
        cout % 8 || cout > 176)
        return VV_ERR_ARG;
    cudaError_t e = cudaSuccess;
    if (!conv3x3_tc((const __half*)x, n, h, w, cin, (const __half*)weights, bias, cout, relu, (__half*)y,
                    (cudaStream_t)stream, &e))
        return VV_ERR_ARG;
    return e == cudaSuccess ? VV_OK : VV_ERR_CUDA;
}

extern "C" vv_status vv_nn_tc_status(int* failed, int clear) {
    if (!failed) return VV_ERR_ARG;
    if (cudaMemcpyFromSymbol(failed, g_tc_status, sizeof(int)) != cudaSuccess) return VV_ERR_CUDA;
    if (clear) {
        int zero = 0;
        if (cudaMemcpyToSymbol(g_tc_status, &zero, sizeof(int)) != cudaSuccess) return VV_ERR_CUDA;
    }
    return VV_OK;
}

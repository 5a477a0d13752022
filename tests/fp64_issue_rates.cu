// FP64 issue rates of GB300 by instruction and operand pattern: independent
// chains on every SM, timed with CUDA events. The FP64-bound kernels of the
// library are adds and multiplies in the reference's order, so their ceiling
// is the DADD / DMUL rate; a DFMA whose three operands are general register
// values issues faster, which is ncu's FP64 peak. Prints one line per pattern
// (G warp instructions per second) and the ratio of the two.
#include <cstdio>
#include <cuda_runtime.h>

template <int OP>
__global__ void chains(double* out, int iters, double p, double q, double r, double s) {
    double a = 1.0 + threadIdx.x * 1e-3, b = 1.5 + blockIdx.x * 1e-4, c = 1.25, d = 1.75;
    for (int i = 0; i < iters; i++) {
        if (OP == 0) {  // DADD, register operands
            a = __dadd_rn(a, p); b = __dadd_rn(b, q); c = __dadd_rn(c, r); d = __dadd_rn(d, s);
        } else if (OP == 1) {  // DMUL, register operands
            a = __dmul_rn(a, p); b = __dmul_rn(b, q); c = __dmul_rn(c, r); d = __dmul_rn(d, s);
        } else {  // DFMA, three general register operands
            a = __fma_rn(a, p, q); b = __fma_rn(b, q, r); c = __fma_rn(c, r, s); d = __fma_rn(d, s, p);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a + b + c + d;
}

int main() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) {
        printf("no device\n");
        return 1;
    }
    const int blocks = sms * 8, threads = 256, iters = 400;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const double P = 0.9999999, Q = 1.0000001, R = 0.99999995, S = 1.00000005;
    const char* names[3] = {"dadd", "dmul", "dfma"};
    double rate[3] = {0, 0, 0};
    for (int op = 0; op < 3; op++) {
        for (int rep = 0; rep < 3; rep++) {  // the last of three runs counts
            cudaEventRecord(e0);
            if (op == 0) chains<0><<<blocks, threads>>>(out, iters, P, Q, R, S);
            if (op == 1) chains<1><<<blocks, threads>>>(out, iters, P, Q, R, S);
            if (op == 2) chains<2><<<blocks, threads>>>(out, iters, P, Q, R, S);
            cudaEventRecord(e1);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            const double warp_insts = (double)blocks * threads / 32 * iters * 4;
            rate[op] = warp_insts / (ms * 1e-3) / 1e9;
        }
        printf("%s %.3f\n", names[op], rate[op]);
    }
    const cudaError_t err = cudaGetLastError();
    printf("dfma_over_dadd %.3f\n", rate[2] / rate[0]);
    printf("%s\n", err == cudaSuccess ? "ok" : cudaGetErrorString(err));
    cudaFree(out);
    return err == cudaSuccess ? 0 : 1;
}

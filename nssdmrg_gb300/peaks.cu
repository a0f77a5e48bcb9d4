// Compute-rate microbenchmark: FP64 FMA (DFMA), FP64 MMA (mma.sync m8n8k4)
// and FP32 FMA (FFMA) throughput of the whole GPU, plus the latency of
// dependent FP64 FMA / FP64 division / FP32 FMA chains in one warp (clock64).
// GB300's HBM and bf16 tensor peaks are measured elsewhere; these are the
// denominators of the FP64 and FP32 CUDA-core kernels' rooflines and the
// facts behind keeping serial FP64 chains off the GPU.  Prints one JSON line.
#include <cstdio>
#include <cuda_runtime.h>
#include <cmath>
__global__ void dfma_k(double* out, int iters){
  double a0=threadIdx.x*1e-3, a1=a0+1, a2=a0+2, a3=a0+3, a4=a0+4,a5=a0+5,a6=a0+6,a7=a0+7;
  const double b=0.999999, c=1e-7;
  for(int i=0;i<iters;i++){
#pragma unroll
    for(int j=0;j<16;j++){ a0=fma(a0,b,c);a1=fma(a1,b,c);a2=fma(a2,b,c);a3=fma(a3,b,c);a4=fma(a4,b,c);a5=fma(a5,b,c);a6=fma(a6,b,c);a7=fma(a7,b,c);} }
  out[blockIdx.x*blockDim.x+threadIdx.x]=a0+a1+a2+a3+a4+a5+a6+a7;
}
__global__ void ffma_k(float* out, int iters){
  float a0=threadIdx.x*1e-3f, a1=a0+1, a2=a0+2, a3=a0+3, a4=a0+4,a5=a0+5,a6=a0+6,a7=a0+7;
  const float b=0.999999f, c=1e-7f;
  for(int i=0;i<iters;i++){
#pragma unroll
    for(int j=0;j<16;j++){ a0=fmaf(a0,b,c);a1=fmaf(a1,b,c);a2=fmaf(a2,b,c);a3=fmaf(a3,b,c);a4=fmaf(a4,b,c);a5=fmaf(a5,b,c);a6=fmaf(a6,b,c);a7=fmaf(a7,b,c);} }
  out[blockIdx.x*blockDim.x+threadIdx.x]=a0+a1+a2+a3+a4+a5+a6+a7;
}
__global__ void dmma_k(double* out, int iters){
  double a=threadIdx.x*1e-3, b=0.5;
  double d0=0,d1=0, e0=0,e1=0, f0=0,f1=0, g0=0,g1=0;
  for(int i=0;i<iters;i++){
#pragma unroll
    for(int j=0;j<16;j++){
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(d0),"+d"(d1) : "d"(a),"d"(b));
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(e0),"+d"(e1) : "d"(a),"d"(b));
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(f0),"+d"(f1) : "d"(a),"d"(b));
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(g0),"+d"(g1) : "d"(a),"d"(b));
    } }
  out[blockIdx.x*blockDim.x+threadIdx.x]=d0+d1+e0+e1+f0+f1+g0+g1;
}
// dependent chains, one warp: cycles per operation
#define LAT_N 2048
__global__ void lat_k(double* dout, float* fout, long long* cyc, int active){
  double x = threadIdx.x*1e-3 + 1.0, y = threadIdx.x*1e-3 + 1.5; float f = threadIdx.x*1e-3f + 1.0f;
  long long t0 = clock64();
  if (threadIdx.x < active) {
#pragma unroll 16
    for (int i = 0; i < LAT_N; ++i) x = fma(x, 0.999, 1e-3);
  }
  long long t1 = clock64();
  if (threadIdx.x < active) {
    for (int i = 0; i < LAT_N / 8; ++i) y = 0.75 / y + 0.5;
  }
  long long t2 = clock64();
  if (threadIdx.x < active) {
#pragma unroll 16
    for (int i = 0; i < LAT_N; ++i) f = fmaf(f, 0.999f, 1e-3f);
  }
  long long t3 = clock64();
  dout[threadIdx.x] = x + y; fout[threadIdx.x] = f;
  if (threadIdx.x == 0) { cyc[0] = t1 - t0; cyc[1] = t2 - t1; cyc[2] = t3 - t2; }
}
int main(){
  int nsm; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  cudaDeviceProp pr; cudaGetDeviceProperties(&pr,0);
  double best_d = 0, best_f = 0, best_m = 0;
  int blocks=nsm*8, threads=256; size_t n=(size_t)blocks*threads;
  double* dout; float* fout; cudaMalloc(&dout,n*8); cudaMalloc(&fout,n*4);
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  int it=2000;
  for(int rep=0;rep<2;rep++){
  dfma_k<<<blocks,threads>>>(dout,10); cudaDeviceSynchronize();
  cudaEventRecord(e0); dfma_k<<<blocks,threads>>>(dout,it); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms,e0,e1);
  best_d = fmax(best_d, 2.0*n*it*16*8/ms/1e6);
  cudaEventRecord(e0); ffma_k<<<blocks,threads>>>(fout,it*4); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms,e0,e1);
  best_f = fmax(best_f, 2.0*n*it*4*16*8/ms/1e6);
  cudaEventRecord(e0); dmma_k<<<blocks,threads>>>(dout,it/4); cudaEventRecord(e1); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms,e0,e1);
  // per warp per mma: 8*8*4*2 = 512 flops
  best_m = fmax(best_m, 512.0*(n/32)*(it/4)*16*4/ms/1e6);
  }
  long long* dcyc; cudaMalloc(&dcyc, 4*sizeof(long long)); long long hc[3] = {0, 0, 0}; double lat[2][3];
  for (int a = 0; a < 2; ++a) {
    for (int rep = 0; rep < 2; ++rep) lat_k<<<1, 32>>>(dout, fout, dcyc, a == 0 ? 1 : 32);
    cudaMemcpy(hc, dcyc, 3*sizeof(long long), cudaMemcpyDeviceToHost);
    lat[a][0] = (double)hc[0] / LAT_N; lat[a][1] = (double)hc[1] / (LAT_N / 8); lat[a][2] = (double)hc[2] / LAT_N;
  }
  cudaError_t e = cudaGetLastError();
  printf("{\"device\": \"%s\", \"sm\": \"%d.%d\", \"sms\": %d, \"dfma_gflops\": %.1f, \"dmma_gflops\": %.1f, "
         "\"ffma_gflops\": %.1f, \"dfma_chain_cycles\": [%.1f, %.1f], \"ddiv_chain_cycles\": [%.1f, %.1f], "
         "\"ffma_chain_cycles\": [%.1f, %.1f], \"chain_lanes\": [1, 32], \"status\": \"%s\"}\n",
         pr.name, pr.major, pr.minor, nsm, best_d, best_m, best_f, lat[0][0], lat[1][0], lat[0][1], lat[1][1],
         lat[0][2], lat[1][2], cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}

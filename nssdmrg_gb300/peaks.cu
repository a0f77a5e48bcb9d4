// Compute-rate microbenchmark: FP64 FMA (DFMA), FP64 MMA (mma.sync m8n8k4),
// FP32 FMA (FFMA) and TF32 tensor-core (tcgen05.mma kind::tf32) throughput of
// the whole GPU, plus the latency of dependent FP64 FMA / FP64 division /
// FP32 FMA chains in one warp (clock64).  GB300's HBM and bf16 tensor peaks
// are measured elsewhere; these are the denominators of the FP64 and FP32
// CUDA-core kernels' rooflines, of the split-TF32 sector GEMM's, and the
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
// tcgen05 kind::tf32 issue rate: one CTA per SM, one thread issues M=128,
// N=256, K=8 MMAs back to back from shared-memory operands (zeros, 128-byte
// swizzled K-major, A 16 KiB, B 32 KiB) into a TMEM accumulator, committing
// to an mbarrier every 64 MMAs.  2*128*256*8 flops per MMA.
__device__ __forceinline__ unsigned long long tf_desc(unsigned saddr) {
  unsigned long long d = (unsigned long long)((saddr & 0x3FFFF) >> 4);
  d |= 1ull << 16; d |= (unsigned long long)(1024 >> 4) << 32; d |= 1ull << 46; d |= 2ull << 61;
  return d;
}
__global__ void __launch_bounds__(128, 1) tf32mma_k(int rounds, int* err){
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char* base = (unsigned char*)(((size_t)tsm + 1023) & ~(size_t)1023);
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ unsigned tbase;
  for (int i = threadIdx.x; i < (48 * 1024) / 16; i += blockDim.x) ((int4*)base)[i] = make_int4(0, 0, 0, 0);
  const unsigned sb0 = (unsigned)__cvta_generic_to_shared(&bar[0]), sb1 = (unsigned)__cvta_generic_to_shared(&bar[1]);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(sb0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(sb1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" :: "r"((unsigned)__cvta_generic_to_shared(&tbase)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (threadIdx.x == 0) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(base), b = a + 16384;
    const unsigned idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
    // round r commits to bar[r & 1]; the thread waits for round r - 1 only,
    // so the tensor core always has the next 64 MMAs queued
    auto wait = [&](int r) -> bool {
      unsigned ok = 0;
      const unsigned sb = (r & 1) ? sb1 : sb0, par = (unsigned)((r >> 1) & 1);
      for (unsigned it = 0; it < (1u << 24) && !ok; ++it)
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(ok) : "r"(sb), "r"(par) : "memory");
      return ok != 0;
    };
    int r = 0;
    for (; r < rounds; ++r) {
      for (int i = 0; i < 64; ++i) {
        const unsigned o = (i & 3) * 32;
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
                     :: "r"(tbase), "l"(tf_desc(a + o)), "l"(tf_desc(b + o)), "r"(idesc), "r"(i > 0 ? 1u : 0u));
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"((r & 1) ? sb1 : sb0) : "memory");
      if (r > 0 && !wait(r - 1)) { atomicExch(err, 1); break; }
    }
    if (r == rounds && r > 0 && !wait(r - 1)) atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" :: "r"(tbase));
}

// L2 read bandwidth: a 48 MiB buffer (L2-resident after the first pass) read
// as float4 by every SM, reps times; the sum keeps the loads alive
__global__ void l2read_k(const float4* __restrict__ x, size_t n4, int reps, float* out){
  float acc = 0.f;
  for (int r = 0; r < reps; ++r)
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
      const float4 v = __ldcg(x + i);
      acc += v.x + v.y + v.z + v.w;
    }
  if (acc == 12345.f) out[0] = acc;
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
  // tcgen05 kind::tf32
  double best_t = 0;
  {
    int* derr; cudaMalloc(&derr, sizeof(int)); cudaMemset(derr, 0, sizeof(int));
    const int smem = 48 * 1024 + 1024, rounds = 400;
    cudaFuncSetAttribute(tf32mma_k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    tf32mma_k<<<nsm, 128, smem>>>(4, derr); cudaDeviceSynchronize();
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0); tf32mma_k<<<nsm, 128, smem>>>(rounds, derr); cudaEventRecord(e1); cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      best_t = fmax(best_t, 2.0 * 128 * 256 * 8 * 64.0 * rounds * nsm / ms / 1e6);
    }
    int herr = 0; cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost);
    if (herr) best_t = 0;
  }
  // L2 read bandwidth
  double best_l2 = 0;
  {
    const size_t bytes = (size_t)48 << 20, n4 = bytes / 16;
    float4* buf; cudaMalloc(&buf, bytes); cudaMemset(buf, 0, bytes);
    const int reps = 40;
    l2read_k<<<nsm * 4, 512>>>(buf, n4, 2, fout); cudaDeviceSynchronize();
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0); l2read_k<<<nsm * 4, 512>>>(buf, n4, reps, fout); cudaEventRecord(e1); cudaEventSynchronize(e1);
      cudaEventElapsedTime(&ms, e0, e1);
      best_l2 = fmax(best_l2, (double)bytes * reps / ms / 1e6);
    }
    cudaFree(buf);
  }
  long long* dcyc; cudaMalloc(&dcyc, 4*sizeof(long long)); long long hc[3] = {0, 0, 0}; double lat[2][3];
  for (int a = 0; a < 2; ++a) {
    for (int rep = 0; rep < 2; ++rep) lat_k<<<1, 32>>>(dout, fout, dcyc, a == 0 ? 1 : 32);
    cudaMemcpy(hc, dcyc, 3*sizeof(long long), cudaMemcpyDeviceToHost);
    lat[a][0] = (double)hc[0] / LAT_N; lat[a][1] = (double)hc[1] / (LAT_N / 8); lat[a][2] = (double)hc[2] / LAT_N;
  }
  cudaError_t e = cudaGetLastError();
  printf("{\"device\": \"%s\", \"sm\": \"%d.%d\", \"sms\": %d, \"dfma_gflops\": %.1f, \"dmma_gflops\": %.1f, "
         "\"ffma_gflops\": %.1f, \"tf32_tc_gflops\": %.1f, \"l2_read_gbs\": %.1f, \"dfma_chain_cycles\": [%.1f, %.1f], \"ddiv_chain_cycles\": [%.1f, %.1f], "
         "\"ffma_chain_cycles\": [%.1f, %.1f], \"chain_lanes\": [1, 32], \"status\": \"%s\"}\n",
         pr.name, pr.major, pr.minor, nsm, best_d, best_m, best_f, best_t, best_l2, lat[0][0], lat[1][0], lat[0][1], lat[1][1],
         lat[0][2], lat[1][2], cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}

// Pipe-rate probe behind the FP64 design decisions: throughput of FP32/FP64
// arithmetic and of the conversions between formats on this GPU, from
// independent dependency chains (ILP 8), timed with CUDA events.
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o pipe_rates pipe_rates.cu && ./pipe_rates
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#define ITERS 2048
#define ILP 8
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)

template<int OP> __global__ void kern(float* outf, double* outd, long long* outl, float seed) {
  int tid = blockIdx.x*blockDim.x+threadIdx.x;
  float f[ILP]; double d[ILP]; long long l[ILP];
  #pragma unroll
  for (int k=0;k<ILP;k++){ f[k]=seed+tid*1e-7f+k; d[k]=f[k]; l[k]=tid+k; }
  for (int it=0; it<ITERS; it++) {
    #pragma unroll
    for (int k=0;k<ILP;k++) {
      if (OP==0) f[k] = fmaf(f[k], 0.999f, 1e-3f);                  // FFMA
      if (OP==1) d[k] = fma(d[k], 0.999, 1e-3);                      // DFMA
      if (OP==2) d[k] = d[k] + 1e-3;                                 // DADD
      if (OP==3) { d[k] = (double)f[k]; f[k] = (float)(d[k]*0.5) ; } // F2F both + DMUL
      if (OP==4) { l[k] = __float2ll_rn(f[k]); f[k] = f[k]*0.999f + (float)(l[k]&1); } // F2I.S64 + I2F32(s32)
      if (OP==5) { d[k] = __ll2double_rn(l[k]); l[k] = l[k] + (long long)(d[k]!=0.0); } // I2F.F64.S64
      if (OP==6) { int t = __float2int_rn(f[k]); f[k] = f[k]*0.999f + (float)(t&1); } // F2I.S32
      if (OP==7) l[k] = l[k] + (l[k]>>7) + 3;                        // int64 add/shift
      if (OP==8) f[k] = sqrtf(f[k]) + 1.0f;                          // sqrtf
      if (OP==9) f[k] = rsqrtf(f[k]) + 1.0f;                         // rsqrt
      if (OP==10) d[k] = d[k] * 0.999;                               // DMUL
      if (OP==11) { float h = (float)d[k]; d[k] = d[k] - (double)h*0.5 + 1.0; } // F2F.F32.F64 + F2F.F64.F32 + DFMA/DADD
      if (OP==12) f[k] = f[k]/ (f[k]+1.0f);                          // fdiv
      if (OP==13) d[k] = 1.0/(d[k]+1.0);                             // ddiv
    }
  }
  float sf=0; double sd=0; long long sl=0;
  #pragma unroll
  for (int k=0;k<ILP;k++){ sf+=f[k]; sd+=d[k]; sl+=l[k]; }
  if (sf==1.2345f || sd==1.2345 || sl==12345) { outf[0]=sf; outd[0]=sd; outl[0]=sl; }
}

template<int OP> int run(const char* name, int opsPerIter, float* f, double* d, long long* l) {
  cudaEvent_t a,b; cudaEventCreate(&a); cudaEventCreate(&b);
  int blocks = 152*8, threads = 256;
  kern<OP><<<blocks,threads>>>(f,d,l,1.0f); CK(cudaDeviceSynchronize());
  cudaEventRecord(a);
  for (int r=0;r<3;r++) kern<OP><<<blocks,threads>>>(f,d,l,1.0f);
  cudaEventRecord(b); CK(cudaEventSynchronize(b));
  float ms; cudaEventElapsedTime(&ms,a,b); ms/=3;
  double ops = (double)blocks*threads*ITERS*ILP*opsPerIter;
  printf("%-28s %8.3f ms  %10.1f Gop/s  (%.1f op/clk/SM at 1.9GHz)\n", name, ms, ops/ms/1e6, ops/ms/1e6/152/1.9);
  return 0;
}
int main(){
  float* f; double* d; long long* l;
  CK(cudaMalloc(&f,64)); CK(cudaMalloc(&d,64)); CK(cudaMalloc(&l,64));
  cudaDeviceProp p; cudaGetDeviceProperties(&p,0); printf("%s SMs=%d cc=%d.%d\n",p.name,p.multiProcessorCount,p.major,p.minor);
  run<0>("FFMA",1,f,d,l); run<1>("DFMA",1,f,d,l); run<2>("DADD",1,f,d,l); run<10>("DMUL",1,f,d,l);
  run<3>("F2F f32->f64 + f64->f32 + DMUL(iter)",1,f,d,l);
  run<11>("F2F pair + DFMA (iter)",1,f,d,l);
  run<4>("F2I.S64 + misc (iter)",1,f,d,l); run<5>("I2F.F64.S64 + misc (iter)",1,f,d,l);
  run<6>("F2I.S32 + misc (iter)",1,f,d,l); run<7>("int64 add+shift (iter)",1,f,d,l);
  run<8>("sqrtf (iter)",1,f,d,l); run<9>("rsqrtf (iter)",1,f,d,l); run<12>("fdiv (iter)",1,f,d,l); run<13>("ddiv (iter)",1,f,d,l);
  return 0;
}

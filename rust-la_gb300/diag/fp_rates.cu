// Diagnostic: issue throughput of this GPU's FP64 and FP32 pipes (DFMA,
// unfused DMUL+DADD, the FP64 mma.sync shapes, FFMA) with register-resident
// independent chains on every SM. The FP64 figures decide how the LU kernels
// are built (FP64 FMA, not the FP64 tensor instruction) and give the FP64
// roofline denominator.
// Build and run: nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp_rates fp_rates.cu && ./fp_rates
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__);return 1;}}while(0)

__global__ void k_dfma(double* out, int iters, double a, double b){
  double r[8];
  #pragma unroll
  for(int i=0;i<8;i++) r[i]=threadIdx.x*1e-3+i;
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<8;i++) r[i]=fma(r[i],a,b);
  }
  double s=0; for(int i=0;i<8;i++) s+=r[i];
  if(s==123.456) out[0]=s;
}
__global__ void k_dmuladd(double* out, int iters, double a, double b){
  double r[8];
  #pragma unroll
  for(int i=0;i<8;i++) r[i]=threadIdx.x*1e-3+i;
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<8;i++) r[i]=__dadd_rn(__dmul_rn(r[i],a),b);
  }
  double s=0; for(int i=0;i<8;i++) s+=r[i];
  if(s==123.456) out[0]=s;
}
__global__ void k_ffma(float* out, int iters, float a, float b){
  float r[16];
  #pragma unroll
  for(int i=0;i<16;i++) r[i]=threadIdx.x*1e-3f+i;
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<16;i++) r[i]=fmaf(r[i],a,b);
  }
  float s=0; for(int i=0;i<16;i++) s+=r[i];
  if(s==123.456f) out[0]=s;
}
// m8n8k4 f64: A 1 reg, B 1 reg, C/D 2 regs per thread. 512 flops per mma.
__global__ void k_dmma884(double* out, int iters){
  double a=threadIdx.x*1e-3, b=1.0-threadIdx.x*1e-4;
  double c[4][2];
  #pragma unroll
  for(int i=0;i<4;i++){c[i][0]=0;c[i][1]=0;}
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<4;i++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
        : "+d"(c[i][0]), "+d"(c[i][1]) : "d"(a), "d"(b));
  }
  double s=0; for(int i=0;i<4;i++) s+=c[i][0]+c[i][1];
  if(s==123.456) out[0]=s;
}
// m16n8k4 f64: A 2 regs, B 1 reg, C/D 4 regs. 1024 flops per mma.
__global__ void k_dmma1684(double* out, int iters){
  double a0=threadIdx.x*1e-3, a1=a0+1, b=1.0-threadIdx.x*1e-4;
  double c[4][4];
  #pragma unroll
  for(int i=0;i<4;i++) for(int j=0;j<4;j++) c[i][j]=0;
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<4;i++)
      asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
        : "+d"(c[i][0]), "+d"(c[i][1]), "+d"(c[i][2]), "+d"(c[i][3]) : "d"(a0), "d"(a1), "d"(b));
  }
  double s=0; for(int i=0;i<4;i++) for(int j=0;j<4;j++) s+=c[i][j];
  if(s==123.456) out[0]=s;
}
// m16n8k16 f64: A 8 regs, B 4 regs, C 4 regs. 4096 flops per mma.
__global__ void k_dmma16816(double* out, int iters){
  double a[8], b[4];
  for(int i=0;i<8;i++) a[i]=threadIdx.x*1e-3+i;
  for(int i=0;i<4;i++) b[i]=1.0-threadIdx.x*1e-4*i;
  double c[2][4];
  #pragma unroll
  for(int i=0;i<2;i++) for(int j=0;j<4;j++) c[i][j]=0;
  for(int it=0;it<iters;it++){
    #pragma unroll
    for(int i=0;i<2;i++)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};"
        : "+d"(c[i][0]), "+d"(c[i][1]), "+d"(c[i][2]), "+d"(c[i][3])
        : "d"(a[0]),"d"(a[1]),"d"(a[2]),"d"(a[3]),"d"(a[4]),"d"(a[5]),"d"(a[6]),"d"(a[7]),
          "d"(b[0]),"d"(b[1]),"d"(b[2]),"d"(b[3]));
  }
  double s=0; for(int i=0;i<2;i++) for(int j=0;j<4;j++) s+=c[i][j];
  if(s==123.456) out[0]=s;
}

template<class F> float timeit(F f){
  cudaEvent_t a,b; cudaEventCreate(&a); cudaEventCreate(&b);
  f(); cudaDeviceSynchronize();
  cudaEventRecord(a); f(); cudaEventRecord(b); cudaEventSynchronize(b);
  float ms; cudaEventElapsedTime(&ms,a,b); return ms;
}
int main(){
  cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,0));
  int sms=p.multiProcessorCount;
  printf("device %s sms %d cc %d.%d\n", p.name, sms, p.major, p.minor);
  double* d; CK(cudaMalloc(&d, 64));
  int it=4096;
  for(int bpsm: {1,2,4,8}) for(int thr: {128,256,512}){
    int blocks=sms*bpsm;
    float ms=timeit([&]{k_dfma<<<blocks,thr>>>(d,it,1.0000001,1e-9);});
    double fl=2.0*8*it*(double)blocks*thr;
    printf("DFMA  bpsm=%d thr=%d: %.3f ms  %.3f TFLOP/s\n",bpsm,thr,ms,fl/ms/1e9);
  }
  CK(cudaGetLastError());
  for(int bpsm: {2,4}){ int thr=256, blocks=sms*bpsm;
    float ms=timeit([&]{k_dmuladd<<<blocks,thr>>>(d,it,1.0000001,1e-9);});
    double fl=2.0*8*it*(double)blocks*thr;
    printf("DMUL+DADD bpsm=%d: %.3f ms  %.3f TFLOP/s (2 flops per pair)\n",bpsm,ms,fl/ms/1e9);
  }
  for(int bpsm: {2,4,8}){ int thr=256, blocks=sms*bpsm;
    float ms=timeit([&]{k_ffma<<<blocks,thr>>>((float*)d,it,1.0000001f,1e-9f);});
    double fl=2.0*16*it*(double)blocks*thr;
    printf("FFMA bpsm=%d: %.3f ms  %.3f TFLOP/s\n",bpsm,ms,fl/ms/1e9);
  }
  CK(cudaGetLastError());
  for(int bpsm: {1,2,4,8}) for(int thr: {128,256}){
    int blocks=sms*bpsm; int iters=1024;
    float ms=timeit([&]{k_dmma884<<<blocks,thr>>>(d,iters);});
    double fl=512.0*4*iters*(double)blocks*(thr/32);
    printf("DMMA m8n8k4 bpsm=%d thr=%d: %.3f ms %.3f TFLOP/s\n",bpsm,thr,ms,fl/ms/1e9);
  }
  CK(cudaGetLastError());
  for(int bpsm: {1,2,4}) for(int thr: {128,256}){
    int blocks=sms*bpsm; int iters=1024;
    float ms=timeit([&]{k_dmma1684<<<blocks,thr>>>(d,iters);});
    double fl=1024.0*4*iters*(double)blocks*(thr/32);
    printf("DMMA m16n8k4 bpsm=%d thr=%d: %.3f ms %.3f TFLOP/s\n",bpsm,thr,ms,fl/ms/1e9);
  }
  CK(cudaGetLastError());
  for(int bpsm: {1,2,4}) for(int thr: {128,256}){
    int blocks=sms*bpsm; int iters=512;
    float ms=timeit([&]{k_dmma16816<<<blocks,thr>>>(d,iters);});
    double fl=4096.0*2*iters*(double)blocks*(thr/32);
    printf("DMMA m16n8k16 bpsm=%d thr=%d: %.3f ms %.3f TFLOP/s\n",bpsm,thr,ms,fl/ms/1e9);
  }
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  return 0;
}

// Throughput probe: DFMA / DADD / DMUL / DDIV / DSQRT / FFMA rates on this GPU.
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("err %s line %d\n",cudaGetErrorString(e),__LINE__); return 1;}}while(0)
template<int OP> __global__ void kd(double* out, double a, double b, int iters){
  double r0=threadIdx.x*1e-9+1.0, r1=r0+1e-3, r2=r0+2e-3, r3=r0+3e-3, r4=r0+4e-3, r5=r0+5e-3, r6=r0+6e-3, r7=r0+7e-3;
  for(int it=0; it<iters; ++it){
    if(OP==0){ r0=fma(r0,a,b); r1=fma(r1,a,b); r2=fma(r2,a,b); r3=fma(r3,a,b); r4=fma(r4,a,b); r5=fma(r5,a,b); r6=fma(r6,a,b); r7=fma(r7,a,b);} 
    if(OP==1){ r0=r0+a; r1=r1+a; r2=r2+a; r3=r3+a; r4=r4+a; r5=r5+a; r6=r6+a; r7=r7+a;}
    if(OP==2){ r0=b/r0; r1=b/r1; r2=b/r2; r3=b/r3; r4=b/r4; r5=b/r5; r6=b/r6; r7=b/r7;}
    if(OP==3){ r0=sqrt(r0+a); r1=sqrt(r1+a); r2=sqrt(r2+a); r3=sqrt(r3+a); r4=sqrt(r4+a); r5=sqrt(r5+a); r6=sqrt(r6+a); r7=sqrt(r7+a);}
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=r0+r1+r2+r3+r4+r5+r6+r7;
}
__global__ void kf(float* out, float a, float b, int iters){
  float r[8]; for(int i=0;i<8;i++) r[i]=threadIdx.x*1e-6f+i;
  for(int it=0; it<iters; ++it){ 
#pragma unroll
    for(int i=0;i<8;i++) r[i]=fmaf(r[i],a,b);}
  float s=0; for(int i=0;i<8;i++) s+=r[i]; out[blockIdx.x*blockDim.x+threadIdx.x]=s;
}
int main(){
  int dev=0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,dev)); int clk=0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);
  printf("name %s SMs %d cc %d.%d smem/block optin %zu L2 %d clock %d kHz\n",p.name,p.multiProcessorCount,p.major,p.minor,p.sharedMemPerBlockOptin,p.l2CacheSize,clk);
  int nb=p.multiProcessorCount*8, nt=256; double* d; float* f; CK(cudaMalloc(&d,nb*nt*8)); CK(cudaMalloc(&f,nb*nt*4));
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  const char* names[4]={"DFMA","DADD","DDIV","DSQRT"};
  for(int op=0;op<4;op++){
    int iters = (op>=2)? 256: 4096;
    for(int rep=0;rep<3;rep++){
      cudaEventRecord(e0);
      if(op==0) kd<0><<<nb,nt>>>(d,0.999999,1e-7,iters);
      if(op==1) kd<1><<<nb,nt>>>(d,1e-7,1e-7,iters);
      if(op==2) kd<2><<<nb,nt>>>(d,1e-7,1.0000001,iters);
      if(op==3) kd<3><<<nb,nt>>>(d,1e-7,1e-7,iters);
      cudaEventRecord(e1); CK(cudaEventSynchronize(e1)); float ms; cudaEventElapsedTime(&ms,e0,e1);
      double nops=(double)nb*nt*iters*8;
      if(rep==2) printf("%s: %.3f ms, %.3f Gop/s (thread-ops), %.1f ops/clk/SM at %d MHz\n",names[op],ms,nops/ms/1e6, nops/(ms*1e-3)/p.multiProcessorCount/(clk*1e3), clk/1000);
    }
  }
  for(int rep=0;rep<3;rep++){
    cudaEventRecord(e0); kf<<<nb,nt>>>(f,0.999f,1e-3f,16384); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    float ms; cudaEventElapsedTime(&ms,e0,e1); double nops=(double)nb*nt*16384*8;
    if(rep==2) printf("FFMA: %.3f ms, %.1f Gop/s\n",ms,nops/ms/1e6);
  }
  CK(cudaGetLastError());
  return 0;
}

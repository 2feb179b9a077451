// Test and benchmark infrastructure (reference arm), never part of the
// library: explicit instantiations of the stablebear reference's own CUDA
// block kernel, sb::internal::cuda_pcf_block_integrate
// (include/sbear/cuda/cuda_pcf_kernel.cuh:95-136, with the rectangle walk of
// lines 36-92 and the operations of include/sbear/functional/operations.cuh),
// compiled from the reference's headers where they lie into a device-only
// cubin (oracle/_ref/ref_kernels.cubin, by oracle/build_oracle.py).
// ref_gpu.cpp loads it through the CUDA driver API and drives it tile by
// tile with the reference's scheduler parameters, so the reference kernel
// can be timed on the same GPU as this library's kernels.
#include "sbear/cuda/cuda_pcf_kernel.cuh"
#include "sbear/functional/operations.cuh"

template __global__ void sb::internal::cuda_pcf_block_integrate<float, float, sb::OperationL1Dist<float, float>>(
    sb::internal::PcfBlockKernelParams<float, float>, float, float, sb::OperationL1Dist<float, float>);
template __global__ void sb::internal::cuda_pcf_block_integrate<float, float, sb::OperationLpDist<float, float>>(
    sb::internal::PcfBlockKernelParams<float, float>, float, float, sb::OperationLpDist<float, float>);
template __global__ void sb::internal::cuda_pcf_block_integrate<float, float, sb::OperationL2InnerProduct<float, float>>(
    sb::internal::PcfBlockKernelParams<float, float>, float, float, sb::OperationL2InnerProduct<float, float>);
template __global__ void sb::internal::cuda_pcf_block_integrate<double, double, sb::OperationL1Dist<double, double>>(
    sb::internal::PcfBlockKernelParams<double, double>, double, double, sb::OperationL1Dist<double, double>);
template __global__ void sb::internal::cuda_pcf_block_integrate<double, double, sb::OperationLpDist<double, double>>(
    sb::internal::PcfBlockKernelParams<double, double>, double, double, sb::OperationLpDist<double, double>);
template __global__ void sb::internal::cuda_pcf_block_integrate<double, double, sb::OperationL2InnerProduct<double, double>>(
    sb::internal::PcfBlockKernelParams<double, double>, double, double, sb::OperationL2InnerProduct<double, double>);

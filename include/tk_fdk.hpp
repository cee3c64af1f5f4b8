// tk_fdk.hpp -- header-only C++ class FilteredBackProjection over the C ABI.
//
// Same class name, method names, argument order and return types as the
// reference engine (Lukas-kV/TomoKvas FBPG/kernel.cuh:82-151), so a driver
// written against the reference (FBPG/para_TC.cpp:130-153) compiles against
// this header instead of kernel.cuh and links with libtk_fdk.so.
//
// The output object passed to SetReconstructionProperties is any class with
// `float *GetBlock(int n, bool collecting)` -- the reference's bin_siz
// (FBPG/mucat_file.h:141-193) fits as is.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <iostream>

#include "tk_fdk.h"

class FilteredBackProjection {
public:
    // pipelined: the reference's call sequence always ends in CalculateReconstruction
    FilteredBackProjection()
    {
        tk_fdk_create(&h_);
        tk_fdk_set_pipeline(h_, 1);
    }
    ~FilteredBackProjection() { tk_fdk_destroy(h_); }
    FilteredBackProjection(const FilteredBackProjection &) = delete;
    FilteredBackProjection &operator=(const FilteredBackProjection &) = delete;

    void SetSinogramProperties(float *_sinogram, const int &_sinogram_X, const float &_centre_X,
                               const int &_sinogram_Y, const int &_sinogram_Z, const float &_centre_Z,
                               const float &_delta_fi, float _distance, float _sampling)
    {
        report(tk_fdk_set_sinogram_properties(h_, _sinogram, _sinogram_X, _centre_X, _sinogram_Y, _sinogram_Z,
                                              _centre_Z, _delta_fi, _distance, _sampling));
    }

    template <class Output>
    void SetReconstructionProperties(Output *_output_file, const int &_reconstruction_X, const float &_centre_X,
                                     const int &_reconstruction_Y, const float &_centre_Y,
                                     const int &_reconstruction_Z, const float &_centre_Z, const float &_rot)
    {
        output_ = _output_file;
        get_block_ = &FilteredBackProjection::call_get_block<Output>;
        report(tk_fdk_set_reconstruction_properties(h_, _reconstruction_X, _centre_X, _reconstruction_Y, _centre_Y,
                                                    _reconstruction_Z, _centre_Z, _rot));
    }

    void SetAxisDirection(const bool &_X = false, const bool &_Y = false, const bool &_Z = false)
    {
        report(tk_fdk_set_axis_direction(h_, _X, _Y, _Z));
    }
    void SetGPUid(const int &_ID = 0) { report(tk_fdk_set_gpu_id(h_, _ID)); }
    void SetBlockSize(const int &_sz = 16) { report(tk_fdk_set_block_size(h_, _sz)); }
    void SetAllocationLimit(const long long int &_memory_limit = (long long int)1024 * 1024 * 1024)
    {
        report(tk_fdk_set_allocation_limit(h_, _memory_limit));
    }
    void SetCollecting(const bool &_collecting = false) { report(tk_fdk_set_collecting(h_, _collecting)); }
    void SetShowInfo(const bool &_show = false) { report(tk_fdk_set_show_info(h_, _show)); }
    void SetScaleXYZ(const float &_scale) { report(tk_fdk_set_scale_xyz(h_, _scale)); }

    cudaError_t Initialize() { return status(tk_fdk_initialize(h_)); }
    cudaError_t CalculateReconstruction()
    {
        if (!output_) return status(TK_ERR_STATE);
        return status(tk_fdk_calculate_reconstruction(h_, get_block_, this));
    }

    // The reference uploads its per-angle sin/cos tables here (kernel.cu:430-471);
    // this engine forms them on the host for every launch (the same FP64 sin/cos
    // of the FP32 angle), so there is nothing to prepare ahead of the call.
    cudaError_t CalcSinCos() { return cudaSuccess; }

    // Device summary on stdout, as kernel.cu:901-913 prints it.
    void fShowInfo() { report(tk_fdk_show_info(h_)); }

    static size_t GetFreeMemInfo(int _GPUId) { return tk_get_free_mem_info(_GPUId); }

    // access to the extensions of the C ABI (filters, storage, raw input)
    tk_fdk *handle() { return h_; }

private:
    template <class Output>
    static float *call_get_block(void *self, int n, int collecting)
    {
        auto *me = static_cast<FilteredBackProjection *>(self);
        return static_cast<Output *>(me->output_)->GetBlock(n, collecting != 0);
    }

    static void report(int rc)
    {
        if (rc != TK_OK) std::cerr << "tk_fdk: " << tk_last_error() << std::endl;
    }

    // Failures are reported on std::cerr and mapped to CUDA error codes, as
    // the reference returns cudaError_t (kernel.cu:336-340).
    static cudaError_t status(int rc)
    {
        if (rc == TK_OK) return cudaSuccess;
        report(rc);
        return rc == TK_ERR_OOM ? cudaErrorMemoryAllocation
               : rc == TK_ERR_INVALID || rc == TK_ERR_STATE ? cudaErrorInvalidValue
                                                             : cudaErrorUnknown;
    }

    tk_fdk *h_ = nullptr;
    void *output_ = nullptr;
    tk_block_sink get_block_ = nullptr;
};

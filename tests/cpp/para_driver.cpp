// para_driver.cpp -- a para_TC-style driver (FBPG/para_TC.cpp:106-155) written
// against the reference interface, compiled here against include/tk_fdk.hpp.
//
// usage: para_driver sino.f32 out.f32 W N H X Y Z zb D tau dfi scale
// Reads a float32 sinogram [H][N][W], reconstructs with the reference call
// sequence and writes the float32 volume [Z][Y][X] block by block through a
// bin_siz-like writer (GetBlock hands out Z slabs of a host buffer).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "tk_fdk.hpp"

struct block_writer {  // stand-in for bin_siz (FBPG/mucat_file.h:141-193)
    std::vector<float> vol;
    size_t slab = 0;
    int zb = 16;
    float *GetBlock(int n, bool) { return vol.data() + (size_t)n * zb * slab; }
};

int main(int argc, char **argv)
{
    if (argc != 14) {
        std::fprintf(stderr, "usage: %s sino out W N H X Y Z zb D tau dfi scale\n", argv[0]);
        return 2;
    }
    const int W = std::atoi(argv[3]), N = std::atoi(argv[4]), H = std::atoi(argv[5]);
    const int X = std::atoi(argv[6]), Y = std::atoi(argv[7]), Z = std::atoi(argv[8]), zb = std::atoi(argv[9]);
    const float D = std::atof(argv[10]), tau = std::atof(argv[11]), dfi = std::atof(argv[12]);
    const float scale = std::atof(argv[13]);
    std::vector<float> data((size_t)W * N * H);
    FILE *f = std::fopen(argv[1], "rb");
    if (!f || std::fread(data.data(), sizeof(float), data.size(), f) != data.size()) return 3;
    std::fclose(f);

    block_writer out;
    out.zb = zb;
    out.slab = (size_t)X * Y;
    out.vol.assign(((size_t)Z + zb) * out.slab, 0.f);

    FilteredBackProjection *FBP = new FilteredBackProjection();
    FBP->SetGPUid(0);
    FBP->SetBlockSize(zb);
    FBP->SetAllocationLimit((long long int)1024 * 1024 * 1024);
    FBP->SetCollecting(false);
    FBP->SetShowInfo(false);
    FBP->SetAxisDirection(false, false, false);
    FBP->SetSinogramProperties(data.data(), W, (W - 1) / 2.f, N, H, ((double)H - 1) / 2., dfi, D, tau);
    FBP->SetReconstructionProperties(&out, X, ((double)X - 1) / 2., Y, ((double)Y - 1) / 2., Z, 0, 0.f);
    FBP->SetScaleXYZ(scale);
    if (FBP->Initialize() != cudaSuccess) {
        delete FBP;
        return 1;
    }
    if (FBP->CalcSinCos() != cudaSuccess) {
        delete FBP;
        return 1;
    }
    FBP->fShowInfo();
    std::vector<float>().swap(data);  // the data now lives on the GPU (para_TC.cpp:150)
    const cudaError_t rc = FBP->CalculateReconstruction();
    delete FBP;
    if (rc != cudaSuccess) return 1;
    f = std::fopen(argv[2], "wb");
    if (!f) return 3;
    std::fwrite(out.vol.data(), sizeof(float), (size_t)Z * out.slab, f);
    std::fclose(f);
    return 0;
}

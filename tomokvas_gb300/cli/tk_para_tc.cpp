// tk_para_tc.cpp -- the reference's command-line driver (FBPG/para_TC.cpp:
// main, 5-176) on Linux over this engine:
//
//   tk_para_tc [--quiet] path/to/scan.CRA
//
// Reads setting.xml from the working directory (written with the defaults
// when missing, as LoadSetting/SaveSetting), the .CRA scan description and
// its raw float32 projections, reconstructs every scan block with the
// FilteredBackProjection call sequence of the reference, and writes
// <scan>.bin / <scan>.siz next to the .CRA through the bin_siz-style block
// writer.  Differences from the reference: projections are handed to the
// engine projection-major as they lie in the raw file (no host transpose);
// a scan block is one angle block (HBM holds it; the engine streams when it
// does not), and the program never waits for Enter unless setting.xml asks.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "tk_fdk.hpp"
#include "tk_io.hpp"

int main(int argc, char **argv)
{
    bool quiet = false;
    std::string cra;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--quiet")) quiet = true;
        else cra = argv[i];
    }
    if (cra.empty()) {
        std::fprintf(stderr, "usage: %s [--quiet] file.CRA\n", argv[0]);
        return 2;
    }
    // path and file name without extension (para_TC.cpp:25-38), either separator
    const size_t sl = cra.find_last_of("/\\");
    const size_t dt = cra.rfind('.');
    const std::string path = sl == std::string::npos ? std::string(".") : cra.substr(0, sl);
    const size_t name0 = sl == std::string::npos ? 0 : sl + 1;
    const std::string filename = cra.substr(name0, (dt == std::string::npos || dt < name0) ? std::string::npos
                                                                                         : dt - name0);

    tk_io::Settings set;
    if (!set.Load("setting.xml")) set.Save("setting.xml");

    tk_io::CraFile datafile(path, filename);
    if (int rc = datafile.GetMetaData()) {
        std::fprintf(stderr, "cannot read %s/%s.CRA (%d)\n", path.c_str(), filename.c_str(), rc);
        return 3;
    }
    unsigned sx, sy, sz, rec_x, rec_y, rec_z;
    datafile.GetSize(sx, sy, sz);
    datafile.GetRecSize(rec_x, rec_y, rec_z);
    const double ReconstructionScale = datafile.GetScale();
    rec_x = (unsigned)(rec_x * ReconstructionScale);  // para_TC.cpp:60-62
    rec_y = (unsigned)(rec_y * ReconstructionScale);
    rec_z = (unsigned)(rec_z * ReconstructionScale);
    const float delta_fi = (float)datafile.GetDFI();
    const float distance = (float)datafile.GetDistance();
    const float sampling = (float)datafile.GetSampling();
    const int ScanBlocks = datafile.GetNumberOfBlocks();
    if (!quiet)
        std::printf("scan %s: %u x %u x %u projections, volume %u x %u x %u, %d scan block(s), D = %g px\n",
                    filename.c_str(), sx, sy, sz, rec_x, rec_y, rec_z, ScanBlocks, distance);

    tk_io::BinSizWriter output_file(path, filename);
    output_file.SetScanBlocksCount(ScanBlocks);
    if (output_file.SetImageSize((int)rec_x, (int)rec_y, (int)rec_z)) {
        std::fprintf(stderr, "cannot create %s/%s.bin\n", path.c_str(), filename.c_str());
        return 3;
    }
    output_file.SetSlicesPerBlock(set.NoOfSlicesInOneBlock);

    std::vector<float> data((size_t)sx * sy * sz);
    const auto t0 = std::chrono::steady_clock::now();
    for (int ScanBlock = 0; ScanBlock < ScanBlocks; ++ScanBlock) {
        datafile.SetActiveBlock(ScanBlock);
        output_file.SetScanBlockOffset(ScanBlock);
        const float centre = (float)datafile.GetCentreOfRotation();
        if (datafile.LoadProjections(data.data())) {
            std::fprintf(stderr, "cannot read the projections of scan block %d\n", ScanBlock);
            return 3;
        }
        const float rot = (float)datafile.GetRotRad();

        FilteredBackProjection *FBP = new FilteredBackProjection();
        FBP->SetGPUid(set.GPUId);
        FBP->SetBlockSize(set.NoOfSlicesInOneBlock);
        FBP->SetAllocationLimit((long long int)set.GPUAllocLimit * 1024 * 1024);
        FBP->SetCollecting(false);
        FBP->SetShowInfo(!quiet && ScanBlock == 0);
        FBP->SetAxisDirection(set.x_direction, set.y_direction, set.z_direction);
        FBP->SetSinogramProperties(data.data(), (int)sx, centre, (int)sy, (int)sz,
                                   ((double)sz - 1) / 2. + set.VerticalCenter, delta_fi, distance,
                                   sampling * 0.0001);  // sampling in cm (para_TC.cpp:139)
        tk_fdk_set_input_layout(FBP->handle(), TK_LAYOUT_PROJECTION);  // frames as read, no transpose
        FBP->SetReconstructionProperties(&output_file, (int)rec_x, ((double)rec_x - 1) / 2., (int)rec_y,
                                         ((double)rec_y - 1) / 2., (int)rec_z, 0, rot);
        FBP->SetScaleXYZ(1. / ReconstructionScale);
        if (FBP->Initialize() != cudaSuccess) {
            delete FBP;
            return 1;
        }
        const cudaError_t rc = FBP->CalculateReconstruction();
        delete FBP;
        if (rc != cudaSuccess) return 1;
        output_file.FlushBuffer();
        if (!quiet) std::printf("scan block %d / %d done\n", ScanBlock + 1, ScanBlocks);
    }
    if (output_file.errors()) {
        std::fprintf(stderr, "%d file IO error(s) writing %s/%s.bin\n", output_file.errors(), path.c_str(),
                     filename.c_str());
        return 3;
    }
    if (!quiet)
        std::printf("total time: %.3f s\n",
                    std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    if (set.WaitForEnter && !quiet) {
        std::printf("press enter\n");
        std::getchar();
    }
    return 0;
}

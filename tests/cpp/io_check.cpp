// io_check.cpp -- exercises include/tk_io.hpp (host only, no GPU) for tests/test_io.py.
//
//   io_check cra DIR NAME BLOCK OUT_PROJ OUT_SINO   -> JSON of the derived geometry; the block's
//                                                     projections [N][H][W] and [H][N][W] to files
//   io_check binsiz DIR NAME X Y Z ZB SCANBLOCKS    -> writes two passes (second one collecting)
//   io_check settings FILE [SAVE_TO]                -> JSON of the parsed settings
//   io_check rsq FILE SINX SINY FIRST LAST RAW DARK FLAT -> JSON of the header and the
//                                                     beam-hardening line; rows FIRST..LAST
//                                                     (raw u16, dark and flat f32) to files
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tk_io.hpp"

static int write_file(const char *path, const std::vector<float> &v)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) return 1;
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    if (!std::strcmp(argv[1], "cra") && argc == 7) {
        tk_io::CraFile c(argv[2], argv[3]);
        const int rc = c.GetMetaData();
        if (rc) {
            std::printf("{\"rc\": %d}\n", rc);
            return 0;
        }
        c.SetActiveBlock(std::atoi(argv[4]));
        unsigned sx, sy, sz, rx, ry, rz;
        c.GetSize(sx, sy, sz);
        c.GetRecSize(rx, ry, rz);
        std::vector<float> a((size_t)sx * sy * sz), b(a.size());
        const int l1 = c.LoadProjections(a.data()), l2 = c.LoadData(b.data());
        if (write_file(argv[5], a) || write_file(argv[6], b)) return 3;
        std::printf("{\"rc\": 0, \"load\": [%d, %d], \"distance\": %.9g, \"dfi\": %.9g, \"rot\": %.17g, "
                    "\"centre\": %.17g, \"sampling\": %.17g, \"scale\": %.17g, \"blocks\": %d, "
                    "\"size\": [%u, %u, %u], \"rec\": [%u, %u, %u], \"raw\": \"%s\", \"clockwise\": %d}\n",
                    l1, l2, c.GetDistance(), c.GetDFI(), c.GetRotRad(), c.GetCentreOfRotation(), c.GetSampling(),
                    c.GetScale(), c.GetNumberOfBlocks(), sx, sy, sz, rx, ry, rz, c.header().raw_file.c_str(),
                    (int)c.header().clockwise);
        return 0;
    }
    if (!std::strcmp(argv[1], "binsiz") && argc == 9) {
        const int X = std::atoi(argv[4]), Y = std::atoi(argv[5]), Z = std::atoi(argv[6]), zb = std::atoi(argv[7]);
        const int sb = std::atoi(argv[8]);
        int errors = 0;
        {
            tk_io::BinSizWriter w(argv[2], argv[3]);
            w.SetScanBlocksCount(sb);
            if (w.SetImageSize(X, Y, Z)) return 3;
            w.SetSlicesPerBlock(zb);
            const int nblk = (Z + zb - 1) / zb;
            for (int s = 0; s < sb; ++s) {
                w.SetScanBlockOffset(s);
                // pass 1: value = 1000 s + z + 0.001 (y X + x) for global slice z
                for (int n = 0; n < nblk; ++n) {
                    float *p = w.GetBlock(n, false);
                    for (int k = 0; k < zb && n * zb + k < Z; ++k)
                        for (int i = 0; i < X * Y; ++i) p[(size_t)k * X * Y + i] = 1000.f * s + (n * zb + k) + 0.001f * i;
                }
                w.FlushBuffer();
                // pass 2, collecting: each block comes back with pass 1's values; add 0.5
                for (int n = 0; n < nblk; ++n) {
                    float *p = w.GetBlock(n, true);
                    for (int k = 0; k < zb && n * zb + k < Z; ++k)
                        for (int i = 0; i < X * Y; ++i) p[(size_t)k * X * Y + i] += 0.5f;
                }
                w.FlushBuffer();
            }
            errors = w.errors();
        }
        std::printf("{\"errors\": %d}\n", errors);
        return 0;
    }
    if (!std::strcmp(argv[1], "rsq") && argc == 10) {
        tk_io::RsqFile r(argv[2], std::atoi(argv[3]), std::atoi(argv[4]));
        if (r.LoadHeader()) {
            std::printf("{\"rc\": -1}\n");
            return 0;
        }
        const unsigned first = (unsigned)std::atoi(argv[5]), last = (unsigned)std::atoi(argv[6]);
        const size_t n = last >= first ? last - first + 1 : 0, W = (size_t)r.sin_x(), N = (size_t)r.sin_y();
        std::vector<uint16_t> raw(n * N * W);
        std::vector<float> dark(n * W), flat(n * W);
        const int lrc = r.Load(first, last, raw.data(), dark.data(), flat.data());
        if (!lrc) {
            FILE *f = std::fopen(argv[7], "wb");
            if (!f) return 3;
            std::fwrite(raw.data(), 2, raw.size(), f);
            std::fclose(f);
            if (write_file(argv[8], dark) || write_file(argv[9], flat)) return 3;
        }
        const tk_io::RsqHeader &h = r.header();
        const tk_io::BeamHardening &b = r.beam_hardening();
        std::printf("{\"rc\": 0, \"load\": %d, \"sinograms\": %llu, \"check\": \"%s\", \"samples\": %d, "
                    "\"projections\": %d, \"dim\": [%d, %d, %d], \"data_offset\": %d, \"energy\": %d, "
                    "\"name\": \"%s\", \"bh_parsed\": %d, \"bh_x\": [%d, %d, %d], \"bh_y\": [%.17g, %.17g, %.17g], "
                    "\"A\": %.17g, \"B\": %.17g}\n",
                    lrc, (unsigned long long)r.NumOfSinograms(), h.check, h.nr_of_samples, h.nr_of_projections,
                    h.dimx_p, h.dimy_p, h.dimz_p, h.data_offset, h.energy, h.name, (int)b.parsed, b.X[0], b.X[1],
                    b.X[2], b.Y[0], b.Y[1], b.Y[2], b.A, b.B);
        return 0;
    }
    if (!std::strcmp(argv[1], "settings") && (argc == 3 || argc == 4)) {
        tk_io::Settings s;
        const bool found = s.Load(argv[2]);
        if (argc == 4) s.Save(argv[3]);
        std::printf("{\"found\": %d, \"GPUId\": %d, \"GPUmemLimit\": %d, \"GPUAllocLimit\": %d, "
                    "\"VerticalCenter\": %.17g, \"NoOfSlicesInOneBlock\": %d, \"x\": %d, \"y\": %d, \"z\": %d, "
                    "\"WaitForEnter\": %d}\n",
                    (int)found, s.GPUId, s.GPUmemLimit, s.GPUAllocLimit, s.VerticalCenter, s.NoOfSlicesInOneBlock,
                    (int)s.x_direction, (int)s.y_direction, (int)s.z_direction, (int)s.WaitForEnter);
        return 0;
    }
    return 2;
}

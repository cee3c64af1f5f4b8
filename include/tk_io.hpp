// tk_io.hpp -- the host-side data formats on either side of the FDK engine,
// portable C++17 (no Win32, no TinyXML), header only:
//
//   tk_io::CraFile       .CRA scan description + raw float32 projections
//                        (cra_con, FBPG/mucat_file.cpp:8-164, 189-277, 287-340)
//   tk_io::BinSizWriter  .bin float32 volume + .siz text header, written by a
//                        background IO thread; float *GetBlock(int, bool) is the
//                        block-sink contract of FilteredBackProjection
//                        (bin_siz, FBPG/mucat_file.cpp:430-793)
//   tk_io::Settings      setting.xml (LoadSetting/SaveSetting, FBPG/para_TC.cpp:180-303)
//   tk_io::RsqFile       Scanco .RSQ raw counts with per-row dark/flat rows and the
//                        beam-hardening line (rsq, FBPG/rsq_load.h:13-59,
//                        FBPG/rsq_load.cpp:68-82, 185-227, 488-548)
//
// The derived scan geometry (distance in pixels, angle step, reconstruction
// size clamps, rotation offset of clockwise scans) is computed with the
// reference's float/int arithmetic, because it decides the sample positions.
#pragma once

#include <cerrno>
#include <cmath>
#include <algorithm>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace tk_io {

inline std::string join_path(const std::string &dir, const std::string &name)
{
    if (dir.empty()) return name;
    const char last = dir.back();
    return (last == '/' || last == '\\') ? dir + name : dir + "/" + name;
}

// ------------------------------------------------------------------ .CRA

struct CraHeader {
    std::string raw_file, source_name;
    double sample_spacing = 0;  // um
    double distance = 0;        // cm
    int detector_x = 0, detector_z = 0, num_of_projections = 0, num_of_blocks = 1;
    int x_dimension = 0, z_dimension = 0;
    double rotate_angle = 0;  // degrees
    bool clockwise = false;
    std::vector<double> centre_of_rotation;  // one per scan block
    double scale = 1.;
};

// A .CRA file: "KEY: value" lines, the keys of cra_con (mucat_file.cpp:12-25).
// The raw file holds num_of_blocks scan blocks one after another, each
// num_of_projections frames of detector_z x detector_x float32.  Clockwise
// scans are stored in decreasing angle order.
class CraFile {
public:
    CraFile(std::string dir, std::string name) : dir_(std::move(dir)), name_(std::move(name)) {}

    // Parses <dir>/<name>.CRA and derives the geometry; 0 on success, -1 when
    // the file cannot be opened (GetMetaData, mucat_file.cpp:74-164).
    int GetMetaData()
    {
        std::ifstream f(join_path(dir_, name_ + ".CRA"));
        if (!f.is_open()) return -1;
        static const char *keys[] = {"FILE NAME:",         "SOURCE NAME:",  "SAMPLE SPACING:",
                                     "DISTANCE:",          "DETECTOR X PIXELS:", "DETECTOR Z PIXELS:",
                                     "NUMBER OF PROJECTIONS:", "X DIMENSION:", "Z DIMENSION:",
                                     "ROTATE ANGLE:",      "CENTRE:",       "NUMBER OF BLOCKS:",
                                     "CLOCKWISE:",         "SCALE:"};
        std::string line;
        while (std::getline(f, line)) {
            if (!line.empty() && line.back() == '\r') line.pop_back();
            for (int k = 0; k < 14; ++k) {
                const size_t n = std::strlen(keys[k]);
                if (line.compare(0, n, keys[k]) != 0) continue;
                std::string v = line.substr(n);
                const size_t a = v.find_first_not_of(" \t");
                v = a == std::string::npos ? std::string() : v.substr(a);
                std::istringstream s(v);
                switch (k) {
                case 0: h_.raw_file = v; break;
                case 1: h_.source_name = v; break;
                case 2: s >> h_.sample_spacing; break;
                case 3: s >> h_.distance; break;
                case 4: s >> h_.detector_x; break;
                case 5: s >> h_.detector_z; break;
                case 6: s >> h_.num_of_projections; break;
                case 7: s >> h_.x_dimension; break;
                case 8: s >> h_.z_dimension; break;
                case 9: s >> h_.rotate_angle; break;
                case 10: {
                    double c = 0;
                    s >> c;
                    h_.centre_of_rotation.push_back(c);
                    break;
                }
                case 11: s >> h_.num_of_blocks; break;
                case 12: h_.clockwise = true; break;  // the key alone marks a clockwise scan
                case 13: s >> h_.scale; break;
                }
            }
        }
        if (h_.num_of_projections <= 0 || h_.detector_x <= 0 || h_.detector_z <= 0 || h_.sample_spacing <= 0)
            return -2;
        if (h_.num_of_blocks < 1) h_.num_of_blocks = 1;
        // float members and int/float mixes as in cra_con (mucat_file.cpp:139-161)
        distance_ = (float)(h_.distance * 10000. / h_.sample_spacing);
        delta_fi_ = (float)(2 * 3.14159265358979323846 / h_.num_of_projections);
        const float phi = std::atan((float)(h_.detector_x / 2) / distance_);
        unsigned tmp = 2u * (unsigned)(int)(distance_ * std::sin(phi) + 1);
        if (h_.x_dimension > (int)tmp || h_.x_dimension < 1) h_.x_dimension = (int)tmp;
        tmp = (unsigned)((distance_ - (float)(h_.x_dimension / 2)) / distance_ * (float)h_.detector_z);
        tmp &= ~1u;
        if (h_.z_dimension > (int)tmp) h_.z_dimension = (int)tmp;
        if (h_.z_dimension < 1) h_.z_dimension = 1;
        return 0;
    }

    const CraHeader &header() const { return h_; }
    double GetDistance() const { return distance_; }  // pixels at the rotation axis
    double GetDFI() const { return delta_fi_; }
    double GetSampling() const { return h_.sample_spacing; }
    double GetScale() const { return h_.scale; }
    int GetNumberOfBlocks() const { return h_.num_of_blocks; }
    int SetActiveBlock(int b)
    {
        active_ = (b >= 0 && b < h_.num_of_blocks) ? b : 0;
        return active_;
    }
    double GetCentreOfRotation() const
    {
        return active_ < (int)h_.centre_of_rotation.size() ? h_.centre_of_rotation[active_] : 0.0;
    }
    // Rotation offset of the whole scan block read at once (GetRotRad,
    // mucat_file.cpp:300-340 with one sinogram block): a clockwise scan is
    // stored reversed and starts one angle step later.
    double GetRotRad() const
    {
        double r = h_.clockwise ? (double)delta_fi_ : 0.0;
        return r + h_.rotate_angle * 3.14159265358979323846 / 180.;
    }
    void GetSize(unsigned &sx, unsigned &sy, unsigned &sz) const
    {
        sx = (unsigned)h_.detector_x;
        sy = (unsigned)h_.num_of_projections;
        sz = (unsigned)h_.detector_z;
    }
    void GetRecSize(unsigned &rx, unsigned &ry, unsigned &rz) const
    {
        rx = ry = (unsigned)(h_.x_dimension == 0 ? h_.detector_x : h_.x_dimension);
        rz = (unsigned)h_.z_dimension;
    }

    // The active scan block's projections, projection-major [N][H][W] in
    // increasing angle order (clockwise scans reversed) -- the layout the
    // engine reads in place (TK_LAYOUT_PROJECTION).  0 on success.
    int LoadProjections(float *out) const { return load(out, false); }
    // The same data in the reference's sinogram-major layout [H][N][W]
    // (LoadData, mucat_file.cpp:189-277).
    int LoadData(float *out) const { return load(out, true); }

private:
    int load(float *out, bool sinogram) const
    {
        const size_t W = (size_t)h_.detector_x, H = (size_t)h_.detector_z, N = (size_t)h_.num_of_projections;
        const size_t frame = W * H;
        FILE *f = std::fopen(join_path(dir_, h_.raw_file).c_str(), "rb");
        if (!f) return -1;
        const unsigned long long off = ((unsigned long long)active_ * N * frame) * sizeof(float);
        if (fseeko(f, (off_t)off, SEEK_SET) != 0) {
            std::fclose(f);
            return -1;
        }
        std::vector<float> tmp(sinogram ? frame : 0);
        for (size_t k = 0; k < N; ++k) {
            const size_t a = h_.clockwise ? N - 1 - k : k;  // angle index of the k-th stored frame
            float *dst = sinogram ? tmp.data() : out + a * frame;
            if (std::fread(dst, sizeof(float), frame, f) != frame) {
                std::fclose(f);
                return -1;
            }
            if (sinogram)
                for (size_t r = 0; r < H; ++r) std::memcpy(out + (r * N + a) * W, dst + r * W, W * sizeof(float));
        }
        std::fclose(f);
        return 0;
    }

    std::string dir_, name_;
    CraHeader h_;
    float distance_ = 0.f, delta_fi_ = 0.f;
    int active_ = 0;
};

// ------------------------------------------------------------------ .RSQ

// The 512-byte header block of an RSQ file (ima_data_type, rsq_load.h:13-48),
// little-endian 32-bit fields at their offsets in the block.
struct RsqHeader {
    char check[17] = {};
    int data_type = 0, nr_of_bytes = 0, nr_of_blocks = 0, patient_index = 0, scanner_id = 0;
    int creation_date[2] = {0, 0};
    int dimx_p = 0, dimy_p = 0, dimz_p = 0, dimx_um = 0, dimy_um = 0, dimz_um = 0;
    int slice_thickness_um = 0, slice_increment_um = 0, slice_1_pos_um = 0;
    int min_data_value = 0, max_data_value = 0, mu_scaling = 0;
    int nr_of_samples = 0, nr_of_projections = 0, scandist_um = 0, scanner_type = 0, sampletime_us = 0;
    int index_measurement = 0, site = 0, reference_line_um = 0, recon_alg = 0;
    char name[41] = {};
    int energy = 0, intensity = 0;
    int data_offset = 0;  // in 512-byte blocks
};

// Beam-hardening correction "Corr at X0 X1 X2: Y0 Y1 Y2" (152 bytes at file
// offset 3432) and its line y = A log(x) + B through the first and third
// points (rsq_load.cpp:538-542).  A and B are the flat-field step's A and B
// (tk_flatfield, tk_fdk_set_projections_u16).
struct BeamHardening {
    int X[3] = {0, 0, 0};
    double Y[3] = {0, 0, 0};
    double A = 1.0, B = 0.0;
    bool parsed = false;
};

inline bool ParseBeamHardening(const char *text, BeamHardening &bh)
{
    BeamHardening t;
    if (std::sscanf(text, "Corr at %d %d %d: %lf %lf %lf", &t.X[0], &t.X[1], &t.X[2], &t.Y[0], &t.Y[1], &t.Y[2]) !=
            6 ||
        t.X[2] == t.X[0])
        return false;
    t.A = (t.Y[2] - t.Y[0]) / (t.X[2] - t.X[0]);
    t.B = t.Y[0] - t.A * t.X[0];
    t.parsed = true;
    bh = t;
    return true;
}

// An RSQ file: the header block, the beam-hardening text, and from
// header_offset (3584, rsq_load.cpp:12) one block per detector row of
// (sin_y + 2) x sin_x uint16 counts: the dark row, the flat row, then the
// row's sin_y projections (rsq_load.cpp:283-325).  The sizes are the
// caller's (the reference's defaults: 1024 x 2000); the number of rows in the
// file follows from its size (rsq_load.cpp:80-82).
class RsqFile {
public:
    explicit RsqFile(std::string path, int sin_x = 1024, int sin_y = 2000,
                     unsigned long long header_offset = 3584)
        : path_(std::move(path)), sin_x_(sin_x), sin_y_(sin_y), offset_(header_offset)
    {
    }

    // Reads the header block, the beam-hardening text and the file size.
    // 0 on success, -1 if the file cannot be read.
    int LoadHeader()
    {
        FILE *f = std::fopen(path_.c_str(), "rb");
        if (!f) return -1;
        unsigned char blk[512];
        char bh[153] = {};
        const bool ok = std::fread(blk, 1, 512, f) == 512 && fseeko(f, 3432, SEEK_SET) == 0 &&
                        std::fread(bh, 1, 152, f) == 152 && fseeko(f, 0, SEEK_END) == 0;
        const long long size = ok ? (long long)ftello(f) : -1;
        std::fclose(f);
        if (!ok || size < 0) return -1;
        file_size_ = (unsigned long long)size;
        auto i32 = [&](int off) {
            int32_t v;
            std::memcpy(&v, blk + off, 4);
            return (int)v;
        };
        RsqHeader h;
        std::memcpy(h.check, blk, 16);
        int *fields1[] = {&h.data_type, &h.nr_of_bytes, &h.nr_of_blocks, &h.patient_index, &h.scanner_id,
                          &h.creation_date[0], &h.creation_date[1]};
        for (int k = 0; k < 7; ++k) *fields1[k] = i32(16 + 4 * k);
        int *fields2[] = {&h.dimx_p, &h.dimy_p, &h.dimz_p, &h.dimx_um, &h.dimy_um, &h.dimz_um,
                          &h.slice_thickness_um, &h.slice_increment_um, &h.slice_1_pos_um, &h.min_data_value,
                          &h.max_data_value, &h.mu_scaling, &h.nr_of_samples, &h.nr_of_projections,
                          &h.scandist_um, &h.scanner_type, &h.sampletime_us, &h.index_measurement, &h.site,
                          &h.reference_line_um, &h.recon_alg};
        for (int k = 0; k < 21; ++k) *fields2[k] = i32(44 + 4 * k);
        std::memcpy(h.name, blk + 128, 40);
        h.energy = i32(168);
        h.intensity = i32(172);
        h.data_offset = i32(508);
        header_ = h;
        ParseBeamHardening(bh, bh_);
        return 0;
    }

    const RsqHeader &header() const { return header_; }
    const BeamHardening &beam_hardening() const { return bh_; }
    int sin_x() const { return sin_x_; }
    int sin_y() const { return sin_y_; }
    // Detector rows in the file (CalculateNumOfSinograms, rsq_load.cpp:80-82).
    unsigned long long NumOfSinograms() const
    {
        const unsigned long long row = (unsigned long long)sin_x_ * (sin_y_ + 2) * 2;
        return file_size_ > offset_ ? (file_size_ - offset_) / row : 0;
    }

    // Detector rows [first, last] (LoadImages(first, last), rsq_load.cpp:185-227):
    // raw counts [n][sin_y][sin_x] (the engine's sinogram-major layout, H = n,
    // N = sin_y, W = sin_x) and each row's dark and flat rows as float
    // [n][sin_x] (the per-pixel maps of tk_fdk_set_projections_u16).  0 on
    // success, -1 on a bad range or a short read.
    int Load(unsigned first, unsigned last, uint16_t *raw, float *dark, float *flat) const
    {
        if (last < first || last >= NumOfSinograms()) return -1;
        const size_t W = (size_t)sin_x_, rows = (size_t)sin_y_ + 2;
        FILE *f = std::fopen(path_.c_str(), "rb");
        if (!f) return -1;
        const unsigned long long off = offset_ + (unsigned long long)first * rows * W * 2;
        if (fseeko(f, (off_t)off, SEEK_SET) != 0) {
            std::fclose(f);
            return -1;
        }
        std::vector<uint16_t> blk(rows * W);
        for (unsigned r = 0; r + first <= last; ++r) {
            if (std::fread(blk.data(), 2, blk.size(), f) != blk.size()) {
                std::fclose(f);
                return -1;
            }
            for (size_t x = 0; x < W; ++x) {
                dark[r * W + x] = (float)blk[x];
                flat[r * W + x] = (float)blk[W + x];
            }
            std::memcpy(raw + (size_t)r * sin_y_ * W, blk.data() + 2 * W, (size_t)sin_y_ * W * 2);
        }
        std::fclose(f);
        return 0;
    }

private:
    std::string path_;
    int sin_x_, sin_y_;
    unsigned long long offset_;
    unsigned long long file_size_ = 0;
    RsqHeader header_;
    BeamHardening bh_;
};

// ------------------------------------------------------------ .bin/.siz

// Volume writer with the bin_siz contract: the .bin file holds
// scan_blocks x Z slices of X*Y float32 (scan blocks one after another along
// z); the .siz file is the text "X Y Z*scan_blocks 0".  GetBlock(n,
// collecting) returns a host buffer of slices_per_block slices for Z block n
// of the active scan block; the buffer returned before it is queued for
// writing on a background thread, so file IO overlaps the next block's
// computation.  With collecting, the buffer comes back holding the block's
// current contents in the file (the partial sum of earlier angle blocks).
// Three buffers rotate, as ALMEM = 3 in the reference.
class BinSizWriter {
public:
    BinSizWriter(std::string dir, std::string name)
        : bin_(join_path(dir, name + ".bin")), siz_(join_path(dir, name + ".siz"))
    {
        worker_ = std::thread([this] { run(); });
    }
    ~BinSizWriter()
    {
        FlushBuffer();
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        worker_.join();
        SaveHeader();
    }
    BinSizWriter(const BinSizWriter &) = delete;
    BinSizWriter &operator=(const BinSizWriter &) = delete;

    void SetScanBlocksCount(int n) { scan_blocks_ = n > 0 ? n : 1; }
    // Creates the .bin file at its full size (zero-filled).
    int SetImageSize(int x, int y, int z)
    {
        x_ = x;
        y_ = y;
        z_ = z;
        FILE *f = std::fopen(bin_.c_str(), "wb");
        if (!f) return errno ? errno : -1;
        const unsigned long long bytes = (unsigned long long)scan_blocks_ * x * y * z * sizeof(float);
        int rc = 0;
        if (bytes && (fseeko(f, (off_t)(bytes - 1), SEEK_SET) != 0 || std::fputc(0, f) == EOF)) rc = -1;
        std::fclose(f);
        return rc;
    }
    void SetSlicesPerBlock(int zb)
    {
        zb_ = zb > 0 ? zb : 16;
        for (auto &b : buf_) b.data.assign((size_t)zb_ * x_ * y_, 0.f);
    }
    void SetScanBlockOffset(int k) { scan_offset_ = k; }
    float GetBufferSize() const { return 3.f * zb_ * x_ * y_ * sizeof(float) / 1024.f / 1024.f; }

    float *GetBlock(int n, bool collecting = false)
    {
        std::unique_lock<std::mutex> lk(m_);
        if (cur_ >= 0) queue_write(cur_);  // the engine is done with the previous block
        // a buffer that is neither queued nor being written
        int pick = -1;
        cv_done_.wait(lk, [&] {
            for (int i = 0; i < 3; ++i)
                if (!buf_[i].busy) {
                    pick = i;
                    return true;
                }
            return false;
        });
        Buf &b = buf_[pick];
        b.block = n;
        b.bytes = block_bytes(n);
        b.offset = block_offset(n);
        cur_ = pick;
        if (collecting) {
            // read after every queued write: the FIFO worker keeps the order
            b.busy = true;
            tasks_.push_back({pick, false});
            cv_.notify_all();
            cv_done_.wait(lk, [&] { return !b.busy; });
        }
        return b.data.data();
    }

    // Writes the last block and waits until the file holds everything.
    void FlushBuffer()
    {
        std::unique_lock<std::mutex> lk(m_);
        if (cur_ >= 0) queue_write(cur_);
        cur_ = -1;
        cv_done_.wait(lk, [&] { return tasks_.empty() && !buf_[0].busy && !buf_[1].busy && !buf_[2].busy; });
    }

    int SaveHeader() const
    {
        FILE *f = std::fopen(siz_.c_str(), "w");
        if (!f) return -1;
        std::fprintf(f, "%d %d %d 0", x_, y_, z_ * scan_blocks_);
        std::fclose(f);
        return 0;
    }
    int errors() const { return errors_; }

private:
    struct Buf {
        std::vector<float> data;
        int block = -1;
        size_t bytes = 0;
        unsigned long long offset = 0;
        bool busy = false;
    };
    struct Task {
        int buf;
        bool write;
    };

    size_t block_bytes(int n) const
    {
        const int slices = std::min(zb_, z_ - n * zb_);
        return slices > 0 ? (size_t)slices * x_ * y_ * sizeof(float) : 0;
    }
    unsigned long long block_offset(int n) const
    {
        return ((unsigned long long)scan_offset_ * z_ + (unsigned long long)n * zb_) * x_ * y_ * sizeof(float);
    }
    void queue_write(int i)
    {
        buf_[i].busy = true;
        tasks_.push_back({i, true});
        cv_.notify_all();
    }
    void run()
    {
        std::unique_lock<std::mutex> lk(m_);
        for (;;) {
            cv_.wait(lk, [&] { return stop_ || !tasks_.empty(); });
            if (tasks_.empty()) return;
            const Task t = tasks_.front();
            Buf &b = buf_[t.buf];
            lk.unlock();
            int err = 0;
            if (b.bytes) {
                FILE *f = std::fopen(bin_.c_str(), "r+b");
                if (!f || fseeko(f, (off_t)b.offset, SEEK_SET) != 0) err = 1;
                else if (t.write) err = std::fwrite(b.data.data(), 1, b.bytes, f) != b.bytes;
                else err = std::fread(b.data.data(), 1, b.bytes, f) != b.bytes;
                if (f) std::fclose(f);
            }
            lk.lock();
            tasks_.pop_front();
            errors_ += err;
            b.busy = false;
            cv_done_.notify_all();
        }
    }

    std::string bin_, siz_;
    int x_ = 0, y_ = 0, z_ = 0, zb_ = 16, scan_blocks_ = 1, scan_offset_ = 0;
    Buf buf_[3];
    int cur_ = -1;
    std::deque<Task> tasks_;
    std::mutex m_;
    std::condition_variable cv_, cv_done_;
    bool stop_ = false;
    int errors_ = 0;
    std::thread worker_;
};

// ------------------------------------------------------------- setting.xml

// The <GPU_FBP> settings of the reference's driver with its defaults
// (FBPG/para_TC.cpp:180-260, FBPG/para_TC.h:20-31).
struct Settings {
    int GPUId = 0;
    int GPUmemLimit = 5 * 1024;  // MiB
    int GPUAllocLimit = 1024;    // MiB
    double VerticalCenter = 0;   // detector vertical centre offset (px)
    int NoOfSlicesInOneBlock = 16;
    bool x_direction = false, y_direction = false, z_direction = false;
    bool WaitForEnter = true;

    // true when <GPU_FBP> was found (missing elements keep their defaults).
    bool Load(const std::string &path)
    {
        std::ifstream f(path);
        if (!f.is_open()) return false;
        std::stringstream ss;
        ss << f.rdbuf();
        const std::string x = ss.str();
        if (x.find("<GPU_FBP") == std::string::npos) return false;
        std::string e;
        if (element(x, "GPU", e)) {
            attr(e, "ID", GPUId);
            attr(e, "MemLimit_MiB", GPUmemLimit);
            attr(e, "AllocLimit_MiB", GPUAllocLimit);
        }
        if (element(x, "RECONSTRUCTION", e)) {
            attr(e, "SimultaneouslyReconstructedSlices", NoOfSlicesInOneBlock);
            battr(e, "X_direction", x_direction);
            battr(e, "Y_direction", y_direction);
            battr(e, "Z_direction", z_direction);
            attr(e, "DetectorVerticalCenterOffset", VerticalCenter);
        }
        if (element(x, "GENERAL", e)) battr(e, "WaitForEnter", WaitForEnter);
        return true;
    }
    bool Save(const std::string &path) const
    {
        FILE *f = std::fopen(path.c_str(), "w");
        if (!f) return false;
        std::fprintf(f, "<GPU_FBP>\n    <GPU ID=\"%d\" MemLimit_MiB=\"%d\" AllocLimit_MiB=\"%d\" />\n", GPUId,
                     GPUmemLimit, GPUAllocLimit);
        std::fprintf(f,
                     "    <RECONSTRUCTION SimultaneouslyReconstructedSlices=\"%d\" X_direction=\"%d\" "
                     "Y_direction=\"%d\" Z_direction=\"%d\" DetectorVerticalCenterOffset=\"%.17g\" />\n",
                     NoOfSlicesInOneBlock, (int)x_direction, (int)y_direction, (int)z_direction, VerticalCenter);
        std::fprintf(f, "    <GENERAL WaitForEnter=\"%d\" />\n</GPU_FBP>\n", (int)WaitForEnter);
        std::fclose(f);
        return true;
    }

private:
    static bool element(const std::string &x, const char *name, std::string &out)
    {
        const std::string open = std::string("<") + name;
        size_t p = 0;
        while ((p = x.find(open, p)) != std::string::npos) {
            const char c = p + open.size() < x.size() ? x[p + open.size()] : '\0';
            if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '/' || c == '>') {
                const size_t e = x.find('>', p);
                out = x.substr(p, e == std::string::npos ? std::string::npos : e - p);
                return true;
            }
            p += open.size();
        }
        return false;
    }
    static bool raw_attr(const std::string &e, const char *name, std::string &v)
    {
        const std::string key = std::string(name) + "=";
        size_t p = 0;
        while ((p = e.find(key, p)) != std::string::npos) {
            if (p > 0 && (e[p - 1] == ' ' || e[p - 1] == '\t' || e[p - 1] == '\n' || e[p - 1] == '\r')) {
                size_t q = p + key.size();
                if (q >= e.size()) return false;
                const char quote = e[q];
                if (quote != '"' && quote != '\'') return false;
                const size_t end = e.find(quote, q + 1);
                if (end == std::string::npos) return false;
                v = e.substr(q + 1, end - q - 1);
                return true;
            }
            p += key.size();
        }
        return false;
    }
    template <typename T> static void attr(const std::string &e, const char *name, T &out)
    {
        std::string v;
        if (!raw_attr(e, name, v)) return;
        std::istringstream s(v);
        T t;
        if (s >> t) out = t;
    }
    // TinyXML's int attribute: 0 is false, anything else true
    static void battr(const std::string &e, const char *name, bool &out)
    {
        int i = 0;
        std::string v;
        if (!raw_attr(e, name, v)) {
            out = false;
            return;
        }
        std::istringstream s(v);
        s >> i;
        out = i != 0;
    }
};

}  // namespace tk_io

// mrf_io.hpp -- the reference's file formats for the command-line tools:
// two-label MRF text files (solveMRF.cu:10-65), the demo t-link ".dat" file
// (Application.cu:17-24) and ASCII PPM images (solveMRF.cu:114-127,
// Application.cu:52-72).  Host-only C++17.
#pragma once

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

namespace gcfg_cli {

// Whole-file integer scanner (any whitespace between values).
class IntReader {
  public:
    explicit IntReader(const std::string &path) {
        FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + path);
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf_.resize((size_t)(n > 0 ? n : 0) + 1);
        const size_t got = n > 0 ? std::fread(buf_.data(), 1, (size_t)n, f) : 0;
        std::fclose(f);
        buf_[got] = '\0';
        p_ = buf_.data();
        path_ = path;
    }
    long long next() {
        char *end = nullptr;
        errno = 0;
        const long long v = std::strtoll(p_, &end, 10);
        if (end == p_ || errno) throw std::runtime_error(path_ + ": expected an integer");
        p_ = end;
        return v;
    }
    void fill(std::vector<int> &dst, size_t n) {
        dst.resize(n);
        for (size_t i = 0; i < n; ++i) dst[i] = (int)next();
    }

  private:
    std::vector<char> buf_;
    const char *p_ = nullptr;
    std::string path_;
};

// A two-label MRF.  hcue[y * W + x] (x < W - 1) is the weight of
// (x, y)-(x + 1, y); vcue[y * W + x] (y < H - 1) that of (x, y)-(x, y + 1).
// As in the reference's loader, the last row of both is 0 and the last
// column of hcue is unset there (0 here).
struct Mrf {
    int W = 0, H = 0;
    std::vector<int> dp, dn, hcue, vcue;
};

inline Mrf read_mrf(const std::string &path) {
    IntReader r(path);
    Mrf m;
    m.W = (int)r.next();
    m.H = (int)r.next();
    const long long labels = r.next();
    if (labels != 2) throw std::runtime_error(path + ": only two-label MRFs are supported");
    if (m.W < 1 || m.H < 1) throw std::runtime_error(path + ": bad size");
    const size_t n = (size_t)m.W * m.H;
    for (size_t i = 0; i < n; ++i) r.next();  // ground truth, unused
    r.fill(m.dp, n);
    r.fill(m.dn, n);
    m.hcue.assign(n, 0);
    m.vcue.assign(n, 0);
    for (int y = 0; y < m.H; ++y)
        for (int x = 0; x + 1 < m.W; ++x) m.hcue[(size_t)y * m.W + x] = (int)r.next();
    for (int y = 0; y + 1 < m.H; ++y)
        for (int x = 0; x < m.W; ++x) m.vcue[(size_t)y * m.W + x] = (int)r.next();
    for (int x = 0; x < m.W; ++x) {
        m.hcue[(size_t)(m.H - 1) * m.W + x] = 0;
        m.vcue[(size_t)(m.H - 1) * m.W + x] = 0;
    }
    return m;
}

// Buffered text output of space-terminated integers.
class IntWriter {
  public:
    explicit IntWriter(FILE *f) : f_(f) { buf_.reserve(1 << 20); }
    ~IntWriter() { flush(); }
    void put(long long v) {
        char tmp[24];
        const int k = std::snprintf(tmp, sizeof tmp, "%lld ", v);
        buf_.append(tmp, (size_t)k);
        if (buf_.size() > (1 << 20)) flush();
    }
    void text(const std::string &s) { buf_ += s; }
    void flush() {
        if (!buf_.empty()) std::fwrite(buf_.data(), 1, buf_.size(), f_);
        buf_.clear();
    }

  private:
    FILE *f_;
    std::string buf_;
};

// "H W", then W*H sink and W*H source t-links.
inline void read_dat(const std::string &path, int &W, int &H, std::vector<int> &dp, std::vector<int> &dn) {
    IntReader r(path);
    H = (int)r.next();
    W = (int)r.next();
    if (W < 1 || H < 1) throw std::runtime_error(path + ": bad size");
    r.fill(dn, (size_t)W * H);
    r.fill(dp, (size_t)W * H);
}

// P3 image (any whitespace); pixels as r, g, b ints, row-major.
inline std::vector<int> read_ppm_ascii(const std::string &path, int &W, int &H) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    char magic[3] = {0, 0, 0};
    int maxv = 0;
    if (std::fscanf(f, "%2s %d %d %d", magic, &W, &H, &maxv) != 4 || std::string(magic) != "P3" || W < 1 ||
        H < 1) {
        std::fclose(f);
        throw std::runtime_error(path + ": not an ASCII PPM");
    }
    std::vector<int> px((size_t)3 * W * H);
    for (size_t i = 0; i < px.size(); ++i) {
        if (std::fscanf(f, "%d", &px[i]) != 1) {
            std::fclose(f);
            throw std::runtime_error(path + ": truncated");
        }
    }
    std::fclose(f);
    return px;
}

// White where label != 0, black elsewhere; the reference's exact bytes.
inline void write_label_ppm(const std::string &path, const std::vector<int> &label, int W, int H) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::string out = "P3 " + std::to_string(W) + " " + std::to_string(H) + " 255 \n";
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) out += label[(size_t)y * W + x] ? "255 255 255 " : "0 0 0 ";
        out += "\n";
    }
    std::fwrite(out.data(), 1, out.size(), f);
    std::fclose(f);
}

// The input colour where label != 0, black elsewhere.
inline void write_overlay_ppm(const std::string &path, const std::vector<int> &label, const std::vector<int> &rgb,
                              int W, int H) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::string out = "P3 " + std::to_string(W) + " " + std::to_string(H) + " 255 \n";
    for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            if (label[i])
                out += std::to_string(rgb[3 * i]) + " " + std::to_string(rgb[3 * i + 1]) + " " +
                       std::to_string(rgb[3 * i + 2]) + " ";
            else
                out += "0 0 0 ";
        }
        out += "\n";
    }
    std::fwrite(out.data(), 1, out.size(), f);
    std::fclose(f);
}

}  // namespace gcfg_cli

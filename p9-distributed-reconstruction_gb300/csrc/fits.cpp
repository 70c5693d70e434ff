// FITS input/output of the reference's data layout (Core/FitsIO.cs, which reads and writes
// through CSharpFITS): the primary HDU of each file holds one big-endian array.
//   uvw.fits    double [baseline][time][3]                 ReadUVW (v is negated, FitsIO.cs:196-218)
//   freq.fits   double [channel]                           ReadFrequencies (:186-191)
//   vis.fits    double [baseline][time][channel][pol][2]   ReadVisibilities: (XX + YY) / norm, pol 0 and 3
//   flags.fits  double [baseline][time][channel][pol]      ReadFlags: flagged where the pol sum != 0
//   images      float or double [rows][cols]               ReadImage / ReadImageDouble / Write<T>
// The C# arrays index the slowest FITS axis first (NAXISn ... NAXIS1).  Decoding is split over
// the host's cores; the reference decodes element by element through boxed arrays.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "p9idg_internal.h"

namespace {

p9idg_status fits_fail(p9idg_status st, const std::string &msg) {
    p9idg::record_last_error(msg);
    return st;
}

struct FitsArray {
    int bitpix = 0;
    std::vector<int64_t> axes;  // NAXIS1 (fastest) first
    int64_t data_offset = 0;
    int64_t count() const {
        int64_t n = axes.empty() ? 0 : 1;
        for (int64_t a : axes) n *= a;
        return n;
    }
};

std::string card_value(const char *card) {
    std::string v(card + 10, 70);
    const size_t slash = v.find('/');
    if (slash != std::string::npos && v.find('\'') == std::string::npos) v = v.substr(0, slash);
    const size_t b = v.find_first_not_of(' '), e = v.find_last_not_of(' ');
    return b == std::string::npos ? std::string() : v.substr(b, e - b + 1);
}

// Parses the primary header (2880-byte blocks of 80-character cards, up to END).
p9idg_status read_header(FILE *f, const char *path, FitsArray &out) {
    char block[2880];
    int naxis = -1;
    bool simple = false, end = false;
    int64_t blocks = 0;
    while (!end) {
        if (std::fread(block, 1, sizeof(block), f) != sizeof(block))
            return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(path) + ": truncated FITS header");
        blocks++;
        for (int c = 0; c < 36 && !end; c++) {
            const char *card = block + 80 * c;
            std::string key(card, 8);
            key.erase(key.find_last_not_of(' ') + 1);
            if (key == "END") {
                end = true;
            } else if (key == "SIMPLE") {
                simple = card_value(card) == "T";
            } else if (key == "BITPIX") {
                out.bitpix = std::atoi(card_value(card).c_str());
            } else if (key == "NAXIS") {
                naxis = std::atoi(card_value(card).c_str());
                if (naxis < 0 || naxis > 999) return fits_fail(P9IDG_INVALID_ARGUMENT, "bad NAXIS");
                out.axes.assign(naxis, 0);
            } else if (key.size() > 5 && key.compare(0, 5, "NAXIS") == 0) {
                const int i = std::atoi(key.c_str() + 5);
                if (i >= 1 && i <= naxis) out.axes[i - 1] = std::atoll(card_value(card).c_str());
            }
        }
        if (blocks > 100000) return fits_fail(P9IDG_INVALID_ARGUMENT, "FITS header without END");
    }
    if (!simple || naxis < 0) return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(path) + ": not a FITS primary HDU");
    for (int64_t a : out.axes)
        if (a < 0) return fits_fail(P9IDG_INVALID_ARGUMENT, "negative FITS axis");
    out.data_offset = blocks * 2880;
    return P9IDG_OK;
}

struct File {
    FILE *f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

p9idg_status open_array(const char *path, File &file, FitsArray &arr) {
    if (!path) return fits_fail(P9IDG_INVALID_ARGUMENT, "null path");
    file.f = std::fopen(path, "rb");
    if (!file.f) return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(path) + ": cannot open");
    return read_header(file.f, path, arr);
}

inline uint64_t bswap64(uint64_t v) { return __builtin_bswap64(v); }
inline uint32_t bswap32(uint32_t v) { return __builtin_bswap32(v); }

// Reads count big-endian doubles starting at element `first` of the data unit.
p9idg_status read_doubles(File &file, const FitsArray &arr, int64_t first, int64_t count, std::vector<double> &out) {
    out.resize(static_cast<size_t>(count));
    if (count == 0) return P9IDG_OK;
    if (std::fseek(file.f, static_cast<long>(arr.data_offset + first * 8), SEEK_SET) != 0 ||
        std::fread(out.data(), 8, static_cast<size_t>(count), file.f) != static_cast<size_t>(count))
        return fits_fail(P9IDG_INVALID_ARGUMENT, "truncated FITS data");
    auto *w = reinterpret_cast<uint64_t *>(out.data());
    const int nthreads = static_cast<int>(std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()),
                                                            std::max<int64_t>(1, count >> 20)));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++)
        pool.emplace_back([=] {
            for (int64_t i = count * t / nthreads; i < count * (t + 1) / nthreads; i++) w[i] = bswap64(w[i]);
        });
    for (auto &th : pool) th.join();
    return P9IDG_OK;
}

template <typename Fn>
void parallel_for(int64_t n, Fn fn) {
    const int nthreads =
        static_cast<int>(std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), std::max<int64_t>(1, n)));
    std::vector<std::thread> pool;
    for (int t = 0; t < nthreads; t++)
        pool.emplace_back([=] {
            for (int64_t i = n * t / nthreads; i < n * (t + 1) / nthreads; i++) fn(i);
        });
    for (auto &th : pool) th.join();
}

p9idg_status need(const FitsArray &arr, int bitpix, size_t naxis, const char *what) {
    if (arr.bitpix != bitpix || arr.axes.size() != naxis)
        return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(what) + ": unexpected FITS array type or rank (BITPIX " +
                                                     std::to_string(arr.bitpix) + ", NAXIS " +
                                                     std::to_string(arr.axes.size()) + ")");
    return P9IDG_OK;
}

}  // namespace

extern "C" {

p9idg_status p9idg_fits_shape(const char *path, int32_t *bitpix, int32_t *naxis, int64_t *axes, int32_t max_axes) {
    if (!bitpix || !naxis || (!axes && max_axes > 0)) return fits_fail(P9IDG_INVALID_ARGUMENT, "null argument");
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st != P9IDG_OK) return st;
    *bitpix = arr.bitpix;
    *naxis = static_cast<int32_t>(arr.axes.size());
    for (int32_t i = 0; i < max_axes && i < *naxis; i++) axes[i] = arr.axes[i];
    return P9IDG_OK;
}

p9idg_status p9idg_fits_read_uvw(const char *path, int32_t from_bl, int32_t to_bl, double *out) {
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st == P9IDG_OK) st = need(arr, -64, 3, "ReadUVW");
    if (st != P9IDG_OK) return st;
    if (!out || arr.axes[0] != 3 || from_bl < 0 || to_bl < from_bl || to_bl > arr.axes[2])
        return fits_fail(P9IDG_INVALID_ARGUMENT, "ReadUVW: bad baseline range or uvw axis");
    const int64_t nt = arr.axes[1], n = static_cast<int64_t>(to_bl - from_bl) * nt * 3;
    std::vector<double> buf;
    if ((st = read_doubles(f, arr, static_cast<int64_t>(from_bl) * nt * 3, n, buf)) != P9IDG_OK) return st;
    parallel_for(n / 3, [&](int64_t i) {
        out[3 * i] = buf[3 * i];
        out[3 * i + 1] = -buf[3 * i + 1];  // the reference flips v
        out[3 * i + 2] = buf[3 * i + 2];
    });
    return P9IDG_OK;
}

p9idg_status p9idg_fits_read_frequencies(const char *path, double *out, int64_t capacity) {
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st == P9IDG_OK) st = need(arr, -64, 1, "ReadFrequencies");
    if (st != P9IDG_OK) return st;
    if (!out || capacity < arr.axes[0]) return fits_fail(P9IDG_INVALID_ARGUMENT, "ReadFrequencies: capacity too small");
    std::vector<double> buf;
    if ((st = read_doubles(f, arr, 0, arr.axes[0], buf)) != P9IDG_OK) return st;
    std::memcpy(out, buf.data(), sizeof(double) * buf.size());
    return P9IDG_OK;
}

p9idg_status p9idg_fits_read_visibilities(const char *path, int32_t from_bl, int32_t to_bl, int32_t nt, int32_t nch,
                                          double norm, double *out) {
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st == P9IDG_OK) st = need(arr, -64, 5, "ReadVisibilities");
    if (st != P9IDG_OK) return st;
    const int64_t ncomp = arr.axes[0], npol = arr.axes[1], fch = arr.axes[2], ft = arr.axes[3], fbl = arr.axes[4];
    if (!out || ncomp < 2 || npol < 4 || from_bl < 0 || to_bl < from_bl || to_bl > fbl || nt < 0 || nt > ft ||
        nch < 0 || nch > fch)
        return fits_fail(P9IDG_INVALID_ARGUMENT, "ReadVisibilities: requested range outside the file's array");
    const int64_t per_bl = ft * fch * npol * ncomp;
    std::vector<double> buf;
    if ((st = read_doubles(f, arr, static_cast<int64_t>(from_bl) * per_bl, static_cast<int64_t>(to_bl - from_bl) * per_bl,
                           buf)) != P9IDG_OK)
        return st;
    const int64_t nrows = static_cast<int64_t>(to_bl - from_bl) * nt;
    parallel_for(nrows, [&](int64_t r) {
        const int64_t b = r / nt, t = r % nt;
        for (int k = 0; k < nch; k++) {
            const double *ch = buf.data() + ((b * ft + t) * fch + k) * npol * ncomp;
            const double *xx = ch, *yy = ch + 3 * ncomp;  // pol 0 (XX) and pol 3 (YY)
            double *o = out + 2 * ((b * nt + t) * nch + k);
            o[0] = (xx[0] + yy[0]) / norm;
            o[1] = (xx[1] + yy[1]) / norm;
        }
    });
    return P9IDG_OK;
}

p9idg_status p9idg_fits_read_flags(const char *path, int32_t from_bl, int32_t to_bl, int32_t nt, int32_t nch,
                                   uint8_t *out) {
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st == P9IDG_OK) st = need(arr, -64, 4, "ReadFlags");
    if (st != P9IDG_OK) return st;
    const int64_t npol = arr.axes[0], fch = arr.axes[1], ft = arr.axes[2], fbl = arr.axes[3];
    if (!out || from_bl < 0 || to_bl < from_bl || to_bl > fbl || nt < 0 || nt > ft || nch < 0 || nch > fch)
        return fits_fail(P9IDG_INVALID_ARGUMENT, "ReadFlags: requested range outside the file's array");
    const int64_t per_bl = ft * fch * npol;
    std::vector<double> buf;
    if ((st = read_doubles(f, arr, static_cast<int64_t>(from_bl) * per_bl, static_cast<int64_t>(to_bl - from_bl) * per_bl,
                           buf)) != P9IDG_OK)
        return st;
    const int64_t nrows = static_cast<int64_t>(to_bl - from_bl) * nt;
    parallel_for(nrows, [&](int64_t r) {
        const int64_t b = r / nt, t = r % nt;
        for (int k = 0; k < nch; k++) {
            const double *p = buf.data() + ((b * ft + t) * fch + k) * npol;
            double sum = 0.0;
            for (int64_t l = 0; l < npol; l++) sum += p[l];
            out[(b * nt + t) * nch + k] = sum == 0 ? 0 : 1;
        }
    });
    return P9IDG_OK;
}

// ReadImage (float, BITPIX -32) / ReadImageDouble (double, -64): [rows][cols]
p9idg_status p9idg_fits_read_image(const char *path, int32_t bitpix, void *out, int64_t capacity) {
    File f;
    FitsArray arr;
    p9idg_status st = open_array(path, f, arr);
    if (st == P9IDG_OK) st = need(arr, bitpix, 2, bitpix == -32 ? "ReadImage" : "ReadImageDouble");
    if (st != P9IDG_OK) return st;
    const int64_t n = arr.count();
    if (!out || capacity < n) return fits_fail(P9IDG_INVALID_ARGUMENT, "image capacity too small");
    const int esz = bitpix == -32 ? 4 : 8;
    if (std::fseek(f.f, static_cast<long>(arr.data_offset), SEEK_SET) != 0 ||
        std::fread(out, esz, static_cast<size_t>(n), f.f) != static_cast<size_t>(n))
        return fits_fail(P9IDG_INVALID_ARGUMENT, "truncated FITS image");
    if (esz == 4) {
        auto *w = static_cast<uint32_t *>(out);
        parallel_for(n, [&](int64_t i) { w[i] = bswap32(w[i]); });
    } else {
        auto *w = static_cast<uint64_t *>(out);
        parallel_for(n, [&](int64_t i) { w[i] = bswap64(w[i]); });
    }
    return P9IDG_OK;
}

// FitsIO.Write<T>(T[,] img) (FitsIO.cs:64-84): a primary HDU with one float (-32) or double (-64) image.
p9idg_status p9idg_fits_write_image(const char *path, int32_t bitpix, const void *data, int32_t rows, int32_t cols) {
    if (!path || !data || rows <= 0 || cols <= 0 || (bitpix != -32 && bitpix != -64))
        return fits_fail(P9IDG_INVALID_ARGUMENT, "invalid argument");
    std::string hdr;
    auto card = [&](const std::string &k, const std::string &v) {
        std::string c = k;
        c.resize(8, ' ');
        c += "= ";
        std::string vv = v;
        if (vv.size() < 20) vv = std::string(20 - vv.size(), ' ') + vv;
        c += vv;
        c.resize(80, ' ');
        hdr += c;
    };
    card("SIMPLE", "T");
    card("BITPIX", std::to_string(bitpix));
    card("NAXIS", "2");
    card("NAXIS1", std::to_string(cols));
    card("NAXIS2", std::to_string(rows));
    card("EXTEND", "T");
    std::string end = "END";
    end.resize(80, ' ');
    hdr += end;
    hdr.resize((hdr.size() + 2879) / 2880 * 2880, ' ');
    File f;
    f.f = std::fopen(path, "wb");
    if (!f.f) return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(path) + ": cannot create");
    const int64_t n = static_cast<int64_t>(rows) * cols;
    const int esz = bitpix == -32 ? 4 : 8;
    std::vector<unsigned char> body(static_cast<size_t>((n * esz + 2879) / 2880 * 2880), 0);
    if (esz == 4) {
        const auto *s = static_cast<const uint32_t *>(data);
        auto *d = reinterpret_cast<uint32_t *>(body.data());
        parallel_for(n, [&](int64_t i) { d[i] = bswap32(s[i]); });
    } else {
        const auto *s = static_cast<const uint64_t *>(data);
        auto *d = reinterpret_cast<uint64_t *>(body.data());
        parallel_for(n, [&](int64_t i) { d[i] = bswap64(s[i]); });
    }
    if (std::fwrite(hdr.data(), 1, hdr.size(), f.f) != hdr.size() ||
        std::fwrite(body.data(), 1, body.size(), f.f) != body.size())
        return fits_fail(P9IDG_INVALID_ARGUMENT, std::string(path) + ": write failed");
    return P9IDG_OK;
}

}  // extern "C"

// pgsvt_cli.cpp — the reference's command-line denoiser (src/PGURE-SVT.cpp)
// on libpgsvt: reads a parameter file and a multi-page TIFF, optionally runs
// the hot-pixel filter, denoises with pgsvt_denoise and writes
// <stem>-CLEANED.tif.
//
//   pgsvt_cli paramfile
//
// Same parameter names, defaults and messages as PGURE-SVT.cpp:36-110, with
// the reference's parameter-file grammar (ParseParameters, utils.hpp:55-92):
// "key : value  # comment", tokens after the colon concatenated up to one
// holding '#'; a token that ends the line gets a trailing space (the
// stream is at its end, so skipping whitespace fails), which makes a bare
// "key : true" read as false, as in the reference.  As in the reference,
// `tolerance` is parsed but the run keeps 1e-7 (PGURE-SVT.cpp:101-106
// assigns it to a shadowing local), and the λ
// start point passed is 0 when optimising.  TIFF I/O is built in (no
// libtiff): baseline, uncompressed, 8- or 16-bit grayscale, strips, either
// byte order; 8-bit frames are widened to 16 bits (the reference reads them
// through a 16-bit scanline buffer).  The output is 16-bit, one strip per
// page, as libtiff writes it for the reference.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "pgsvt.h"

namespace {

using Clock = std::chrono::steady_clock;
double secs(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double>(b - a).count();
}

// ParseParameters (utils.hpp:55-92)
std::map<std::string, std::string> parse_parameters(std::istream& in) {
  std::map<std::string, std::string> opts;
  for (std::string line; std::getline(in, line);) {
    std::istringstream iss(line);
    std::string id, eq, val, tok;
    if (!(iss >> id) || id[0] == '#') continue;
    if (!(iss >> eq) || eq == ":" || iss.get() != EOF) {
      while (iss >> tok) {
        if (tok.find('#') != std::string::npos) break;
        if (iss >> std::ws) val += tok;
        else val += tok + " ";
      }
    }
    opts[id] = val;
  }
  return opts;
}

bool str_to_bool(std::string s) {  // StrToBool (utils.hpp:48-53)
  std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return std::tolower(c); });
  return s == "1" || s == "true";
}

// ---- minimal baseline TIFF reader / writer

struct Tiff {
  uint32_t width = 0, height = 0;
  uint16_t bits = 0;
  std::vector<std::vector<uint16_t>> pages;  // row-major frames
};

struct Reader {
  std::vector<unsigned char> b;
  bool le = true;
  uint16_t u16(size_t o) const {
    if (o + 2 > b.size()) throw std::runtime_error("truncated TIFF");
    return le ? (uint16_t)(b[o] | b[o + 1] << 8) : (uint16_t)(b[o] << 8 | b[o + 1]);
  }
  uint32_t u32(size_t o) const {
    if (o + 4 > b.size()) throw std::runtime_error("truncated TIFF");
    return le ? (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 |
                    (uint32_t)b[o + 3] << 24
              : (uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 |
                    (uint32_t)b[o + 3];
  }
  // value(s) of a tag entry: SHORT or LONG, inline or at an offset
  std::vector<uint32_t> values(size_t e) const {
    const uint16_t type = u16(e + 2);
    const uint32_t count = u32(e + 4);
    const size_t sz = type == 3 ? 2 : 4;
    size_t at = e + 8;
    if (sz * count > 4) at = u32(e + 8);
    std::vector<uint32_t> v(count);
    for (uint32_t k = 0; k < count; ++k) v[k] = type == 3 ? u16(at + 2 * k) : u32(at + 4 * k);
    return v;
  }
};

Tiff read_tiff(const std::string& path, uint32_t first, uint32_t last) {  // pages [first, last)
  std::ifstream f(path, std::ios::binary);
  Reader r;
  r.b.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
  if (r.b.size() < 8) throw std::runtime_error("not a TIFF file");
  if (r.b[0] == 'I' && r.b[1] == 'I') r.le = true;
  else if (r.b[0] == 'M' && r.b[1] == 'M') r.le = false;
  else throw std::runtime_error("not a TIFF file");
  if (r.u16(2) != 42) throw std::runtime_error("not a TIFF file (BigTIFF is not read)");
  Tiff t;
  uint32_t off = r.u32(4), page = 0;
  while (off && page < last) {
    const uint16_t n = r.u16(off);
    uint32_t w = 0, h = 0, bits = 1, comp = 1, spp = 1, rps = 0xffffffffu;
    std::vector<uint32_t> so, sb;
    for (uint16_t k = 0; k < n; ++k) {
      const size_t e = off + 2 + 12 * (size_t)k;
      const uint16_t tag = r.u16(e);
      switch (tag) {
        case 256: w = r.values(e)[0]; break;
        case 257: h = r.values(e)[0]; break;
        case 258: bits = r.values(e)[0]; break;
        case 259: comp = r.values(e)[0]; break;
        case 273: so = r.values(e); break;
        case 277: spp = r.values(e)[0]; break;
        case 278: rps = r.values(e)[0]; break;
        case 279: sb = r.values(e); break;
        default: break;
      }
    }
    if (page >= first) {
      if (comp != 1) throw std::runtime_error("compressed TIFF pages are not read");
      if (spp != 1) throw std::runtime_error("only single-channel TIFF pages are read");
      if (t.pages.empty()) {
        t.width = w;
        t.height = h;
        t.bits = (uint16_t)bits;
      } else if (w != t.width || h != t.height || bits != t.bits) {
        throw std::runtime_error("TIFF pages differ in size or depth");
      }
      if (bits != 8 && bits != 16) {
        t.pages.emplace_back();  // depth reported by the caller
        break;
      }
      std::vector<uint16_t> img((size_t)w * h);
      const size_t bps = bits / 8, row = (size_t)w * bps;
      const uint32_t rows_per = std::min(rps, h);
      for (uint32_t y = 0; y < h; ++y) {
        const uint32_t s = y / rows_per, yy = y % rows_per;
        if (s >= so.size()) throw std::runtime_error("TIFF strip table too short");
        const size_t base = (size_t)so[s] + (size_t)yy * row;
        if (base + row > r.b.size()) throw std::runtime_error("truncated TIFF strip");
        for (uint32_t x = 0; x < w; ++x)
          img[(size_t)y * w + x] = bits == 8 ? r.b[base + x] : r.u16(base + 2 * x);
      }
      t.pages.push_back(std::move(img));
    }
    off = r.u32(off + 2 + 12 * (size_t)n);
    ++page;
  }
  return t;
}

void put16(std::vector<unsigned char>& o, uint16_t v) {
  o.push_back(v & 0xff);
  o.push_back(v >> 8);
}
void put32(std::vector<unsigned char>& o, uint32_t v) {
  for (int k = 0; k < 4; ++k) o.push_back((v >> (8 * k)) & 0xff);
}

// little-endian, one strip per page, 16-bit grayscale
void write_tiff(const std::string& path, uint32_t w, uint32_t h,
                const std::vector<std::vector<uint16_t>>& pages) {
  std::vector<unsigned char> o;
  o.insert(o.end(), {'I', 'I'});
  put16(o, 42);
  put32(o, 8);
  const uint32_t nimg = (uint32_t)pages.size();
  for (uint32_t p = 0; p < nimg; ++p) {
    const uint16_t ntag = 11;
    const uint32_t ifd = (uint32_t)o.size();
    const uint32_t data = ifd + 2 + 12 * ntag + 4;
    const uint32_t bytes = w * h * 2;
    const uint32_t next = p + 1 < nimg ? data + bytes : 0;
    put16(o, ntag);
    auto tag = [&](uint16_t t, uint16_t type, uint32_t count, uint32_t v) {
      put16(o, t);
      put16(o, type);
      put32(o, count);
      if (type == 3 && count == 1) {
        put16(o, (uint16_t)v);
        put16(o, 0);
      } else {
        put32(o, v);
      }
    };
    tag(254, 4, 1, 2);                                // NewSubfileType: page
    tag(256, 4, 1, w);                                // ImageWidth
    tag(257, 4, 1, h);                                // ImageLength
    tag(258, 3, 1, 16);                               // BitsPerSample
    tag(259, 3, 1, 1);                                // Compression: none
    tag(262, 3, 1, 1);                                // Photometric: min-is-black
    tag(273, 4, 1, data);                             // StripOffsets
    tag(274, 3, 1, 1);                                // Orientation: top-left
    tag(277, 3, 1, 1);                                // SamplesPerPixel
    tag(278, 4, 1, h);                                // RowsPerStrip
    tag(279, 4, 1, bytes);                            // StripByteCounts
    put32(o, next);
    for (uint16_t v : pages[p]) put16(o, v);
  }
  std::ofstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("cannot open " + path);
  f.write((const char*)o.data(), (std::streamsize)o.size());
  if (!f) throw std::runtime_error("cannot write " + path);
}

uint16_t to_u16(double v) {  // output conversion: truncation, clamped
  if (!(v > 0.0)) return 0;
  if (v >= 65535.0) return 65535;
  return (uint16_t)v;
}

int fail(const std::string& m) {
  std::cerr << "**ERROR**\n" << m << "\n";
  return -1;
}

}  // namespace

int main(int argc, char** argv) {
  std::cout << "PGURE-SVT Denoising (GB300)\n";
  if (argc != 2) {
    std::cout << "  Usage: " << argv[0] << " paramfile\n";
    return -1;
  }
  std::ifstream pf(argv[1]);
  if (!pf) return fail(std::string("Parameter file ") + argv[1] + " not found");
  auto opts = parse_parameters(pf);
  if (!opts.count("filename") || !opts.count("start_frame") || !opts.count("end_frame"))
    return fail("Required parameters not specified\n"
                "You must specify 'filename', 'start_frame' and 'end_frame'");
  try {
    auto geti = [&](const char* k, long d) { return opts.count(k) ? std::stol(opts.at(k)) : d; };
    auto getd = [&](const char* k, double d) { return opts.count(k) ? std::stod(opts.at(k)) : d; };
    auto getb = [&](const char* k, bool d) { return opts.count(k) ? str_to_bool(opts.at(k)) : d; };
    const std::string filename = opts.at("filename");
    const std::string stem = filename.substr(0, filename.find_last_of('.'));
    const long start = std::stol(opts.at("start_frame")), end = std::stol(opts.at("end_frame"));
    if (start < 1 || end < start) return fail("start_frame and end_frame must satisfy 1 <= start <= end");
    const uint32_t nImages = (uint32_t)(end - start + 1);
    pgsvt_params p;
    pgsvt_default_params(&p);
    p.block_size = (uint32_t)geti("patch_size", 4);
    p.traj_length = (uint32_t)geti("trajectory_length", 15);
    p.motion_window = (uint32_t)geti("motion_neighbourhood", 7);
    p.median_size = geti("median_filter", 5);
    p.block_overlap = (uint32_t)geti("patch_overlap", 1);
    p.noise_method = (uint32_t)geti("noise_method", 4);
    p.max_iter = (uint32_t)geti("max_iter", 1000);
    p.n_jobs = geti("n_jobs", -1);
    p.alpha = getd("noise_alpha", -1.0);
    p.mu = getd("noise_mu", -1.0);
    p.sigma = getd("noise_sigma", -1.0);
    const double hot = opts.count("hot_pixel") ? (double)std::stoi(opts.at("hot_pixel")) : -1.0;
    p.random_seed = geti("random_seed", -1);
    p.exp_weighting = getb("exponential_weighting", true);
    const bool normalize = getb("normalize", false);
    p.motion_estimation = getb("motion_estimation", true);
    p.optimize_pgure = getb("optimize_pgure", true);
    p.lambda = 0.0;
    if (!p.optimize_pgure) {
      if (!opts.count("lambda"))
        return fail("PGURE optimization is turned OFF but no lambda specified in parameter file");
      p.lambda = std::stod(opts.at("lambda"));
    }
    p.tol = 1e-7;

    auto t0 = Clock::now();
    const std::string inName = stem + ".tif";
    if (!std::ifstream(inName)) return fail("File " + inName + " not found");
    Tiff t = read_tiff(inName, (uint32_t)(start - 1), (uint32_t)end);
    if (t.width != t.height)
      return fail("Frame dimensions are not square, got " + std::to_string(t.width) + "x" +
                  std::to_string(t.height));
    if (t.bits != 8 && t.bits != 16)
      return fail("Images must be 8-bit or 16-bit, got " + std::to_string(t.bits) + "-bit depth");
    if (nImages > t.pages.size())
      return fail("Sequence only has " + std::to_string(t.pages.size()) + " frames, expected " +
                  std::to_string(nImages));
    // column-major cube, rows = image rows (PGURE-SVT.cpp:142-152)
    const uint32_t S = t.width;
    const size_t F = (size_t)S * S;
    std::vector<uint16_t> X(F * nImages);
    for (uint32_t k = 0; k < nImages; ++k)
      for (uint32_t y = 0; y < S; ++y)
        for (uint32_t x = 0; x < S; ++x) X[k * F + y + (size_t)x * S] = t.pages[k][(size_t)y * S + x];
    auto t1 = Clock::now();
    std::printf("TIFF import:     %10.4f seconds\n", secs(t0, t1));
    if (hot >= 0.0) {
      t0 = Clock::now();
      if (pgsvt_hot_pixel_filter(X.data(), S, S, nImages, hot) != PGSVT_OK)
        return fail(pgsvt_last_error());
      t1 = Clock::now();
      std::printf("Outlier filter:  %10.4f seconds\n", secs(t0, t1));
    }
    t0 = Clock::now();
    std::vector<double> Y(F * nImages), est((size_t)nImages * 4);
    pgsvt_status st;
    const int rc = pgsvt_denoise(X.data(), PGSVT_U16, S, S, nImages, Y.data(), est.data(), &p, &st);
    if (rc != PGSVT_OK) return fail(st.message);
    t1 = Clock::now();
    std::printf("PGURE-SVT:       %10.4f seconds\n", secs(t0, t1));
    t0 = Clock::now();
    if (normalize) {  // to [0, 65535] (PGURE-SVT.cpp:196-199)
      const auto mm = std::minmax_element(Y.begin(), Y.end());
      const double lo = *mm.first, hi = *mm.second;
      for (double& v : Y) v = 65535.0 * (v - lo) / (hi - lo);
    }
    std::vector<std::vector<uint16_t>> out(nImages, std::vector<uint16_t>(F));
    for (uint32_t k = 0; k < nImages; ++k)
      for (uint32_t y = 0; y < S; ++y)
        for (uint32_t x = 0; x < S; ++x) out[k][(size_t)y * S + x] = to_u16(Y[k * F + y + (size_t)x * S]);
    const std::string outName = stem + "-CLEANED.tif";
    write_tiff(outName, S, S, out);
    t1 = Clock::now();
    std::printf("TIFF export:     %10.4f seconds\n\n", secs(t0, t1));
    std::cerr << "Output file:    " << outName << "\n";
  } catch (const std::exception& e) {
    return fail(e.what());
  }
  return 0;
}

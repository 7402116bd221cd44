// mosaic.hpp -- C++ mirror of the mosaic-rust crate's public API for the tile
// matching-and-placement path, over the C ABI of libmosaic_gpu.so
// (include/mosaic_gpu.h).  Header-only, C++17.
//
// Names, argument meaning and results follow the crate:
//   MosaicGenerator / MosaicGeneratorImpl   lib.rs:52-123
//   UsageTracker                            lib.rs:57-89
//   SimilarityDatabase                      similarity.rs:30-138
//   calculate_lab_distance                  similarity.rs:141-146
//   GridPosition                            adjacency.rs:5-46
//   AdjacencyPenaltyCalculator              adjacency.rs:48-214
//   OptimizationConfig / MosaicOptimizer /
//   OptimizationResult                      optimizer.rs:7-221
//   ColorAdjustment /
//   calculate_optimal_adjustment            color_adjustment.rs:6-154
//   generate_mosaic                         main.rs:105-164 + 477-685
//   open_image / open_png / save_png /      main.rs:492, 548, 672 (image::open
//   save_jpeg / save_image                  + to_rgb8, DynamicImage::save)
//   read_material_files                     main.rs:166-206 (load_tiles' files)
//   generate_mosaic_files                   main.rs:105-164 + 477-685 from paths
// plus RAII handles for the resident palette, batches and the request loop.
//
// Error behaviour: where the crate returns Option the mirror returns
// std::optional; where it returns anyhow::Result (file I/O) or where the device
// fails, the mirror throws mosaic::Error carrying the library's status code and
// message.  The library itself never throws, aborts or unwinds.
//
// Differences a caller can observe, all at edges the crate leaves undefined or
// nondeterministic:
//  - Annealing draws from a seeded Philox stream (OptimizationConfig::seed,
//    ::stream) instead of the crate's unseeded thread_rng, so runs repeat.
//  - The optimiser works on palette indices: every tile placed in a grid it
//    optimises must be in the similarity database (Error otherwise).
//  - save_to_file writes a binary file (JSON for a 20 000-tile database is
//    several GB); load_from_file reads that format.
//  - The adjacency functions need build_similarities to have run over every
//    tile added (Error with MG_ERR_STATE otherwise); the crate would look pairs
//    up in a missing or stale matrix.
#pragma once

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mosaic_gpu.h"

namespace mosaic {

using Path = std::filesystem::path;
using Grid = std::vector<std::vector<std::optional<Path>>>;

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

namespace detail {
inline void check(int status) {
  if (status != MG_OK) {
    const char* m = mg_last_error();
    throw Error(status, std::string("mosaic_gpu: ") + (m ? m : "error ") + " (status " + std::to_string(status) + ")");
  }
}
}  // namespace detail

// ---- context -------------------------------------------------------------------------
// One CUDA stream of the library.  The crate has no such object; every mirror
// function takes an optional Context and otherwise uses default_context()
// (device 0, or the device named by MOSAIC_GPU_DEVICE).
class Context {
 public:
  explicit Context(int device = 0) { detail::check(mg_ctx_create(device, &h_)); }
  ~Context() {
    if (h_) mg_ctx_destroy(h_);
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  mg_ctx* get() const { return h_; }
  void sync() { detail::check(mg_ctx_sync(h_)); }
  // How k-nearest queries search (MG_NEAREST_AUTO / _SCAN / _GRID; identical results).
  void set_nearest_method(int method) { detail::check(mg_ctx_set_nearest_method(h_, method)); }
  // How the greedy placement scores candidates: MG_SCORING_CLI (main.rs:335-418)
  // or MG_SCORING_GUI (gui/app_full.rs:1396-1470, the GUI generator).
  void set_scoring(int scoring) { detail::check(mg_ctx_set_scoring(h_, scoring)); }

 private:
  mg_ctx* h_ = nullptr;
};

inline Context& default_context() {
  static Context ctx([] {
    const char* d = std::getenv("MOSAIC_GPU_DEVICE");
    return d ? std::atoi(d) : 0;
  }());
  return ctx;
}

// ---- colours and images ----------------------------------------------------------------
struct Lab {  // palette::Lab<D65, f32>
  float l = 0.0f, a = 0.0f, b = 0.0f;
};
struct Rgb {  // image::Rgb<u8>
  uint8_t r = 0, g = 0, b = 0;
};
// A borrowed RGB8 image (DynamicImage after to_rgb8()).
struct RgbImageView {
  const uint8_t* data = nullptr;
  int width = 0, height = 0;
  int64_t stride = 0;  // bytes between rows; 0 -> 3*width
  int64_t row_bytes() const { return stride ? stride : 3 * (int64_t)width; }
};
struct RgbImage {
  int width = 0, height = 0;
  std::vector<uint8_t> pixels;  // height x width x 3
  RgbImageView view() const { return {pixels.data(), width, height, 3 * (int64_t)width}; }
};

// ---- image files: PNG and JPEG at the two ends of the path --------------------------------------
// PNG data held in memory as RGB8 (image::load_from_memory + to_rgb8).
inline RgbImage decode_png(const uint8_t* data, size_t n) {
  RgbImage img;
  detail::check(mg_png_info(data, n, &img.width, &img.height));
  img.pixels.resize((size_t)img.width * img.height * 3);
  detail::check(mg_png_decode(data, n, img.pixels.data(), 3 * (int64_t)img.width));
  return img;
}
// PNG or JPEG data held in memory, told apart by its signature.
inline RgbImage decode_image(const uint8_t* data, size_t n) {
  RgbImage img;
  detail::check(mg_image_info(data, n, &img.width, &img.height));
  img.pixels.resize((size_t)img.width * img.height * 3);
  detail::check(mg_image_decode(data, n, img.pixels.data(), 3 * (int64_t)img.width));
  return img;
}
namespace detail {
inline std::vector<uint8_t> read_file(const Path& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(MG_ERR_ARG, "cannot open " + path.string());
  return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}
}  // namespace detail
// main.rs:492, 548: image::open(path)?.to_rgb8() for a PNG or JPEG file.
inline RgbImage open_image(const Path& path) {
  const std::vector<uint8_t> data = detail::read_file(path);
  return decode_image(data.data(), data.size());
}
// The same for a file that must be PNG.
inline RgbImage open_png(const Path& path) {
  const std::vector<uint8_t> data = detail::read_file(path);
  return decode_png(data.data(), data.size());
}

// The file half of main.rs:166-206 load_tiles: the regular files of `dir` with
// a png/jpg/jpeg/webp extension (any case), decoded on up to `threads` host
// threads (<= 0: all).  A file that cannot be read or decoded (webp among
// them: no decoder here) is listed in `errors` and skipped, as load_tiles
// prints and skips it.  Files are taken in path order (read_dir's order is
// the file system's).  The aspect filter and its fallback then run on the
// decoded images (mg_select_palette); the crate's fallback would also count
// the skipped files among its first 2 * max_materials entries.
struct MaterialFiles {
  std::vector<Path> paths;
  std::vector<RgbImage> images;
  std::vector<std::pair<Path, std::string>> errors;
  std::vector<RgbImageView> views() const {
    std::vector<RgbImageView> v;
    for (const RgbImage& i : images) v.push_back(i.view());
    return v;
  }
};
inline MaterialFiles read_material_files(const Path& dir, int threads = 0) {
  std::vector<Path> found;
  std::error_code ec;
  for (std::filesystem::directory_iterator it(dir, ec), end; !ec && it != end; it.increment(ec)) {
    if (!it->is_regular_file()) continue;
    std::string ext = it->path().extension().string();
    for (char& c : ext) c = (char)std::tolower((unsigned char)c);
    if (ext == ".png" || ext == ".jpg" || ext == ".jpeg" || ext == ".webp") found.push_back(it->path());
  }
  if (ec) throw Error(MG_ERR_ARG, "cannot read directory " + dir.string() + ": " + ec.message());
  std::sort(found.begin(), found.end());
  MaterialFiles out;
  std::vector<std::vector<uint8_t>> data;
  std::vector<Path> readable;
  for (const Path& p : found) {
    std::ifstream f(p, std::ios::binary);
    if (!f) {
      out.errors.emplace_back(p, "cannot open");
      continue;
    }
    data.emplace_back((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    readable.push_back(p);
  }
  const int n = (int)data.size();
  std::vector<RgbImage> imgs((size_t)n);
  std::vector<const uint8_t*> ptrs((size_t)n);
  std::vector<size_t> lens((size_t)n);
  std::vector<uint8_t*> outs((size_t)n);
  std::vector<int64_t> strides((size_t)n);
  std::vector<int> status((size_t)n, MG_OK);
  uint8_t dummy[3];
  for (int i = 0; i < n; ++i) {
    ptrs[i] = data[i].data();
    lens[i] = data[i].size();
    if (mg_image_info(ptrs[i], lens[i], &imgs[i].width, &imgs[i].height) == MG_OK) {
      imgs[i].pixels.resize((size_t)imgs[i].width * imgs[i].height * 3);
      outs[i] = imgs[i].pixels.data();
      strides[i] = 3 * (int64_t)imgs[i].width;
    } else {  // the decode reports the defect for this file
      outs[i] = dummy;
      strides[i] = 3;
    }
  }
  if (n) mg_image_decode_batch(ptrs.data(), lens.data(), n, outs.data(), strides.data(), threads, status.data());
  for (int i = 0; i < n; ++i) {
    if (status[i] == MG_OK) {
      out.paths.push_back(readable[i]);
      out.images.push_back(std::move(imgs[i]));
    } else {
      out.errors.emplace_back(readable[i], "not a readable PNG or JPEG image (status " + std::to_string(status[i]) + ")");
    }
  }
  return out;
}

// An RGB8 image as PNG file data: level 0 stores the filtered rows, level 1
// codes each 64 KB block with its own Huffman code; `threads` <= 0: all.
inline std::vector<uint8_t> encode_png(const RgbImageView& img, int level = 1, int threads = 0) {
  std::vector<uint8_t> out(mg_png_encode_bound(img.width, img.height));
  size_t len = 0;
  detail::check(mg_png_encode(img.data, img.width, img.height, img.row_bytes(), level, threads, out.data(),
                              out.size(), &len));
  out.resize(len);
  return out;
}
// main.rs:672: DynamicImage::save(path) for a .png path.
inline void save_png(const RgbImageView& img, const Path& path, int level = 1, int threads = 0) {
  const std::vector<uint8_t> data = encode_png(img, level, threads);
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f || !f.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)data.size()))
    throw Error(MG_ERR_ARG, "cannot write " + path.string());
}

// main.rs:672 for a .jpg / .jpeg path: image's JPEG encoder (quality 75 by
// default); this library's baseline encoder (mg_jpeg_encode).
inline std::vector<uint8_t> encode_jpeg(const RgbImageView& img, int quality = 75, int threads = 0) {
  std::vector<uint8_t> out(mg_jpeg_encode_bound(img.width, img.height));
  size_t len = 0;
  detail::check(mg_jpeg_encode(img.data, img.width, img.height, img.row_bytes(), quality, threads, out.data(),
                               out.size(), &len));
  out.resize(len);
  return out;
}
inline void save_jpeg(const RgbImageView& img, const Path& path, int quality = 75, int threads = 0) {
  const std::vector<uint8_t> data = encode_jpeg(img, quality, threads);
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f || !f.write(reinterpret_cast<const char*>(data.data()), (std::streamsize)data.size()))
    throw Error(MG_ERR_ARG, "cannot write " + path.string());
}
// main.rs:672 output_img.save(path): the format from the extension (any
// case): .png (level 1) or .jpg / .jpeg (quality 75); other formats throw.
inline void save_image(const RgbImageView& img, const Path& path, int threads = 0) {
  std::string ext = path.extension().string();
  for (char& c : ext) c = (char)std::tolower((unsigned char)c);
  if (ext == ".png") save_png(img, path, 1, threads);
  else if (ext == ".jpg" || ext == ".jpeg") save_jpeg(img, path, 75, threads);
  else throw Error(MG_ERR_ARG, "only PNG and JPEG output is written: " + path.string());
}

// similarity.rs:141-146
inline float calculate_lab_distance(const Lab& a, const Lab& b) {
  const float x[3] = {a.l, a.a, a.b}, y[3] = {b.l, b.a, b.b};
  return mg_lab_distance(x, y);
}

// ---- lib.rs --------------------------------------------------------------------------
// lib.rs:93-123 (the MosaicGenerator trait's one implementation)
struct MosaicGeneratorImpl {
  // Mean of the per-pixel Lab colours (not the Lab of the mean RGB).
  static Lab calculate_average_lab(const RgbImageView& img, Context& ctx = default_context()) {
    float lab[3];
    detail::check(mg_average_lab(ctx.get(), img.data, img.width, img.height, img.row_bytes(), lab));
    return {lab[0], lab[1], lab[2]};
  }
  static bool is_aspect_ratio_match(float img_aspect, float target_aspect, float tolerance) {
    return mg_is_aspect_ratio_match(img_aspect, target_aspect, tolerance) != 0;
  }
};

// lib.rs:57-89.  Host bookkeeping, as in the crate (the device walk keeps its
// own counters).
class UsageTracker {
 public:
  explicit UsageTracker(size_t max_usage_per_image) : max_(max_usage_per_image) {}
  bool can_use_image(const Path& p) const { return get_usage_count(p) < max_; }
  void use_image(const Path& p) { counts_[p] = get_usage_count(p) + 1; }
  size_t get_usage_count(const Path& p) const {
    auto it = counts_.find(p);
    return it == counts_.end() ? 0 : it->second;
  }
  void reset() { counts_.clear(); }

 private:
  std::map<Path, size_t> counts_;
  size_t max_;
};

// ---- similarity.rs ---------------------------------------------------------------------
namespace detail {
// A small JSON reader and writer for the crate's similarity database files
// (serde_json of similarity.rs:31-41).  Numbers keep their text, so that a
// float is converted once (strtof: the exact f32 the crate wrote) and an index
// as an integer.
struct Json {
  enum Kind { kNull, kBool, kNum, kStr, kArr, kObj } kind = kNull;
  bool b = false;
  std::string text;  // a number's token, or a string's decoded UTF-8
  std::vector<Json> arr;
  std::vector<std::pair<std::string, Json>> obj;
  const Json* get(const std::string& key) const {
    for (const auto& kv : obj)
      if (kv.first == key) return &kv.second;
    return nullptr;
  }
};

class JsonReader {
 public:
  JsonReader(const std::string& s, const Path& file) : p_(s.data()), e_(s.data() + s.size()), file_(file) {}
  Json document() {
    Json v = value(0);
    ws();
    if (p_ != e_) fail("trailing characters");
    return v;
  }

 private:
  const char* p_;
  const char* e_;
  const Path& file_;
  [[noreturn]] void fail(const char* what) { throw Error(MG_ERR_ARG, std::string("JSON: ") + what + ": " + file_.string()); }
  void ws() {
    while (p_ != e_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
  }
  bool take(char c) {
    ws();
    if (p_ != e_ && *p_ == c) {
      ++p_;
      return true;
    }
    return false;
  }
  static void utf8(std::string& out, uint32_t cp) {
    if (cp < 0x80) {
      out += (char)cp;
    } else if (cp < 0x800) {
      out += (char)(0xC0 | cp >> 6);
      out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      out += (char)(0xE0 | cp >> 12);
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | cp >> 18);
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }
  uint32_t hex4() {
    if (e_ - p_ < 4) fail("short \\u escape");
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i, ++p_) {
      const char c = *p_;
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  std::string string() {
    if (!take('"')) fail("string expected");
    std::string out;
    for (;;) {
      if (p_ == e_) fail("unterminated string");
      const char c = *p_++;
      if (c == '"') return out;
      if ((unsigned char)c < 0x20) fail("control character in a string");
      if (c != '\\') {
        out += c;
        continue;
      }
      if (p_ == e_) fail("unterminated string");
      const char x = *p_++;
      switch (x) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          uint32_t cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00) {  // a surrogate pair
            if (e_ - p_ < 2 || p_[0] != '\\' || p_[1] != 'u') fail("lone surrogate");
            p_ += 2;
            const uint32_t lo = hex4();
            if (lo < 0xDC00 || lo > 0xDFFF) fail("bad surrogate pair");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          } else if (cp >= 0xDC00 && cp < 0xE000) {
            fail("lone surrogate");
          }
          utf8(out, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
  }
  Json value(int depth) {
    if (depth > 64) fail("nested too deeply");
    ws();
    if (p_ == e_) fail("value expected");
    Json v;
    const char c = *p_;
    if (c == '{') {
      ++p_;
      v.kind = Json::kObj;
      if (take('}')) return v;
      do {
        std::string k = string();
        if (!take(':')) fail("':' expected");
        v.obj.emplace_back(std::move(k), value(depth + 1));
      } while (take(','));
      if (!take('}')) fail("'}' expected");
    } else if (c == '[') {
      ++p_;
      v.kind = Json::kArr;
      if (take(']')) return v;
      do v.arr.push_back(value(depth + 1));
      while (take(','));
      if (!take(']')) fail("']' expected");
    } else if (c == '"') {
      v.kind = Json::kStr;
      v.text = string();
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      const char* b = p_;
      while (p_ != e_ && (std::isdigit((unsigned char)*p_) || *p_ == '-' || *p_ == '+' || *p_ == '.' || *p_ == 'e' ||
                          *p_ == 'E'))
        ++p_;
      v.kind = Json::kNum;
      v.text.assign(b, p_);
    } else if (e_ - p_ >= 4 && std::strncmp(p_, "true", 4) == 0) {
      p_ += 4;
      v.kind = Json::kBool;
      v.b = true;
    } else if (e_ - p_ >= 5 && std::strncmp(p_, "false", 5) == 0) {
      p_ += 5;
      v.kind = Json::kBool;
    } else if (e_ - p_ >= 4 && std::strncmp(p_, "null", 4) == 0) {
      p_ += 4;
    } else {
      fail("unexpected character");
    }
    return v;
  }
};

inline float json_f32(const Json& v, const Path& file) {
  if (v.kind != Json::kNum) throw Error(MG_ERR_ARG, "JSON: number expected: " + file.string());
  char* end = nullptr;
  const float f = std::strtof(v.text.c_str(), &end);
  if (end != v.text.c_str() + v.text.size()) throw Error(MG_ERR_ARG, "JSON: bad number: " + file.string());
  return f;
}
inline uint64_t json_index(const std::string& t, const Path& file) {
  char* end = nullptr;
  const unsigned long long v = t.empty() || t[0] == '-' ? 0 : std::strtoull(t.c_str(), &end, 10);
  if (t.empty() || t[0] == '-' || end != t.c_str() + t.size()) throw Error(MG_ERR_ARG, "JSON: bad index: " + file.string());
  return v;
}
inline void json_string(std::string& out, const std::string& s) {
  out += '"';
  for (const unsigned char c : s) {
    if (c == '"') out += "\\\"";
    else if (c == '\\') out += "\\\\";
    else if (c == '\n') out += "\\n";
    else if (c == '\r') out += "\\r";
    else if (c == '\t') out += "\\t";
    else if (c < 0x20) {
      char b[8];
      std::snprintf(b, sizeof(b), "\\u%04x", c);
      out += b;
    } else {
      out += (char)c;
    }
  }
  out += '"';
}
inline void json_f32_text(std::string& out, float f) {
  char b[32];
  std::snprintf(b, sizeof(b), "%.9g", (double)f);  // nine digits: strtof gives back the same f32
  out += b;
  if (!std::strpbrk(b, ".eEn")) out += ".0";
}
}  // namespace detail

class SimilarityDatabase {
 public:
  SimilarityDatabase() = default;

  // similarity.rs:61-66; the index is the insertion order.
  void add_tile(const Path& path, const Lab& lab) {
    const size_t index = labs_.size();
    path_to_index_[path] = index;
    index_to_path_[index] = path;
    labs_.push_back(lab);
  }

  // similarity.rs:69-82: every pair i < j, strict upper triangle in row order,
  // computed on the device.
  void build_similarities(Context& ctx = default_context()) {
    const size_t n = labs_.size();
    sims_.assign(n > 1 ? n * (n - 1) / 2 : 0, 0.0f);
    built_n_ = n;
    if (n < 2) return;
    detail::check(mg_similarity_build(ctx.get(), flat_lab().data(), (int)n, MG_SIM_TRIANGULAR, sims_.data()));
  }

  // similarity.rs:85-103: None when a path is unknown or the pair has no entry.
  std::optional<float> get_similarity(const Path& a, const Path& b) const {
    auto ia = path_to_index_.find(a), ib = path_to_index_.find(b);
    if (ia == path_to_index_.end() || ib == path_to_index_.end()) return std::nullopt;
    if (ia->second == ib->second) return 0.0f;
    size_t i = ia->second, j = ib->second;
    if (i > j) std::swap(i, j);
    const size_t n = labs_.size();
    const size_t pos = i * n - i * (i + 1) / 2 + j - i - 1;
    if (pos >= sims_.size()) return std::nullopt;
    return sims_[pos];
  }

  // similarity.rs:106-109
  std::optional<Lab> get_lab_color(const Path& p) const {
    auto it = path_to_index_.find(p);
    if (it == path_to_index_.end() || it->second >= labs_.size()) return std::nullopt;
    return labs_[it->second];
  }

  // similarity.rs:112-116 (the crate writes JSON; this writes the binary format
  // described below).  Throws Error on I/O failure.
  void save_to_file(const Path& file) const {
    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    if (!f) throw Error(MG_ERR_ARG, "cannot create " + file.string());
    const uint64_t n = labs_.size(), ns = sims_.size();
    f.write(kMagic, 8);
    put<uint32_t>(f, kVersion);
    put<uint64_t>(f, n);
    put<uint64_t>(f, ns);
    for (uint64_t i = 0; i < n; ++i) {
      const std::string s = index_to_path_.at(i).generic_string();
      put<uint32_t>(f, (uint32_t)s.size());
      f.write(s.data(), (std::streamsize)s.size());
    }
    for (const Lab& c : labs_) {
      put<float>(f, c.l);
      put<float>(f, c.a);
      put<float>(f, c.b);
    }
    if (ns) f.write(reinterpret_cast<const char*>(sims_.data()), (std::streamsize)(ns * sizeof(float)));
    if (!f) throw Error(MG_ERR_ARG, "write failed: " + file.string());
  }

  // similarity.rs:112-116 in the crate's own format: the serde JSON of its
  // four fields (path_to_index, index_to_path, lab_colors, similarities), so a
  // database written here can be read by the crate.  Throws Error on I/O failure.
  void save_json(const Path& file) const {
    std::string o = "{\n  \"path_to_index\": {";
    const size_t n = labs_.size();
    for (size_t i = 0; i < n; ++i) {
      o += i ? ",\n    " : "\n    ";
      detail::json_string(o, index_to_path_.at(i).generic_string());
      o += ": " + std::to_string(i);
    }
    o += n ? "\n  },\n  \"index_to_path\": {" : "},\n  \"index_to_path\": {";
    for (size_t i = 0; i < n; ++i) {
      o += i ? ",\n    \"" : "\n    \"";
      o += std::to_string(i) + "\": ";
      detail::json_string(o, index_to_path_.at(i).generic_string());
    }
    o += n ? "\n  },\n  \"lab_colors\": [" : "},\n  \"lab_colors\": [";
    for (size_t i = 0; i < n; ++i) {
      o += i ? ",\n    {\n      \"l\": " : "\n    {\n      \"l\": ";
      detail::json_f32_text(o, labs_[i].l);
      o += ",\n      \"a\": ";
      detail::json_f32_text(o, labs_[i].a);
      o += ",\n      \"b\": ";
      detail::json_f32_text(o, labs_[i].b);
      o += "\n    }";
    }
    o += n ? "\n  ],\n  \"similarities\": [" : "],\n  \"similarities\": [";
    for (size_t i = 0; i < sims_.size(); ++i) {
      o += i ? ",\n    " : "\n    ";
      detail::json_f32_text(o, sims_[i]);
    }
    o += sims_.empty() ? "]\n}" : "\n  ]\n}";
    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    if (!f) throw Error(MG_ERR_ARG, "cannot create " + file.string());
    f.write(o.data(), (std::streamsize)o.size());
    if (!f) throw Error(MG_ERR_ARG, "write failed: " + file.string());
  }

  // similarity.rs:119-123.  Reads the binary format below or the crate's JSON
  // (a file whose first non-blank character is '{'), so the crate's existing
  // database files load unchanged.  Throws Error when the file is missing or
  // malformed.
  static SimilarityDatabase load_from_file(const Path& file) {
    std::ifstream f(file, std::ios::binary);
    if (!f) throw Error(MG_ERR_ARG, "cannot open " + file.string());
    char magic[8];
    f.read(magic, 8);
    if (!f || std::memcmp(magic, kMagic, 8) != 0) {
      const std::vector<uint8_t> bytes = detail::read_file(file);
      size_t k = 0;
      while (k < bytes.size() && (bytes[k] == ' ' || bytes[k] == '\t' || bytes[k] == '\n' || bytes[k] == '\r')) ++k;
      if (k < bytes.size() && bytes[k] == '{') return load_json(std::string(bytes.begin(), bytes.end()), file);
      throw Error(MG_ERR_ARG, "not a similarity database: " + file.string());
    }
    if (get<uint32_t>(f, file) != kVersion) throw Error(MG_ERR_ARG, "unsupported version: " + file.string());
    const uint64_t n = get<uint64_t>(f, file), ns = get<uint64_t>(f, file);
    if (ns != 0 && ns != n * (n - 1) / 2) throw Error(MG_ERR_ARG, "inconsistent sizes: " + file.string());
    SimilarityDatabase db;
    std::vector<Path> paths(n);
    for (uint64_t i = 0; i < n; ++i) {
      const uint32_t len = get<uint32_t>(f, file);
      std::string s(len, '\0');
      f.read(s.data(), len);
      if (!f) throw Error(MG_ERR_ARG, "truncated file: " + file.string());
      paths[i] = Path(s);
    }
    for (uint64_t i = 0; i < n; ++i) {
      Lab c;
      c.l = get<float>(f, file);
      c.a = get<float>(f, file);
      c.b = get<float>(f, file);
      db.add_tile(paths[i], c);
    }
    db.sims_.resize(ns);
    if (ns) f.read(reinterpret_cast<char*>(db.sims_.data()), (std::streamsize)(ns * sizeof(float)));
    if (!f) throw Error(MG_ERR_ARG, "truncated file: " + file.string());
    db.built_n_ = ns ? n : 0;
    return db;
  }

  // The crate's JSON layout: lab_colors gives the tiles in index order,
  // index_to_path (or else path_to_index) their paths, similarities the strict
  // upper triangle as the crate holds it (any length; lookups past it find
  // nothing, as similarity.rs:98-102).
  static SimilarityDatabase load_json(const std::string& text, const Path& file) {
    using detail::Json;
    const Json root = detail::JsonReader(text, file).document();
    const Json* labs = root.get("lab_colors");
    const Json* i2p = root.get("index_to_path");
    const Json* p2i = root.get("path_to_index");
    const Json* sims = root.get("similarities");
    if (root.kind != Json::kObj || !labs || labs->kind != Json::kArr || !sims || sims->kind != Json::kArr ||
        ((!i2p || i2p->kind != Json::kObj) && (!p2i || p2i->kind != Json::kObj)))
      throw Error(MG_ERR_ARG, "not a similarity database: " + file.string());
    const size_t n = labs->arr.size();
    std::vector<std::optional<std::string>> paths(n);
    if (i2p && i2p->kind == Json::kObj) {
      for (const auto& kv : i2p->obj) {
        const uint64_t i = detail::json_index(kv.first, file);
        if (i >= n || kv.second.kind != Json::kStr || paths[i]) throw Error(MG_ERR_ARG, "bad index_to_path: " + file.string());
        paths[i] = kv.second.text;
      }
    } else {
      for (const auto& kv : p2i->obj) {
        if (kv.second.kind != Json::kNum) throw Error(MG_ERR_ARG, "bad path_to_index: " + file.string());
        const uint64_t i = detail::json_index(kv.second.text, file);
        if (i >= n || paths[i]) throw Error(MG_ERR_ARG, "bad path_to_index: " + file.string());
        paths[i] = kv.first;
      }
    }
    SimilarityDatabase db;
    for (size_t i = 0; i < n; ++i) {
      const Json& c = labs->arr[i];
      const Json *l = c.get("l"), *a = c.get("a"), *b = c.get("b");
      if (!paths[i] || c.kind != Json::kObj || !l || !a || !b) throw Error(MG_ERR_ARG, "bad lab_colors: " + file.string());
      db.add_tile(Path(*paths[i]), Lab{detail::json_f32(*l, file), detail::json_f32(*a, file), detail::json_f32(*b, file)});
    }
    db.sims_.reserve(sims->arr.size());
    for (const Json& v : sims->arr) db.sims_.push_back(detail::json_f32(v, file));
    db.built_n_ = n >= 2 && db.sims_.size() == n * (n - 1) / 2 ? n : 0;
    return db;
  }

  // similarity.rs:126-138 (same messages on stdout).
  static SimilarityDatabase load_or_new(const Path& file) {
    try {
      SimilarityDatabase db = load_from_file(file);
      std::printf("Loaded similarity database from \"%s\"\n", file.string().c_str());
      return db;
    } catch (const Error&) {
      std::printf("Creating new similarity database\n");
      return SimilarityDatabase();
    }
  }

  // Index view for the device calls (no counterpart in the crate).
  size_t len() const { return labs_.size(); }
  std::optional<size_t> index_of(const Path& p) const {
    auto it = path_to_index_.find(p);
    if (it == path_to_index_.end()) return std::nullopt;
    return it->second;
  }
  const Path& path_of(size_t i) const { return index_to_path_.at(i); }
  // True when build_similarities covered every tile added so far.
  bool built() const { return built_n_ == labs_.size() && !labs_.empty(); }
  std::vector<float> flat_lab() const {
    std::vector<float> v(3 * labs_.size());
    for (size_t i = 0; i < labs_.size(); ++i) {
      v[3 * i] = labs_[i].l;
      v[3 * i + 1] = labs_[i].a;
      v[3 * i + 2] = labs_[i].b;
    }
    return v;
  }
  const std::vector<float>& similarities() const { return sims_; }

 private:
  // File layout (little-endian): "MGSIMDB1", u32 version, u64 n, u64 number of
  // similarity entries (0 or n(n-1)/2), n x (u32 length + UTF-8 path), n x 3
  // f32 Lab, then the strict upper triangle in row order as f32.
  static constexpr char kMagic[9] = "MGSIMDB1";
  static constexpr uint32_t kVersion = 1;
  template <class T>
  static void put(std::ofstream& f, T v) {
    f.write(reinterpret_cast<const char*>(&v), sizeof(T));
  }
  template <class T>
  static T get(std::ifstream& f, const Path& file) {
    T v;
    f.read(reinterpret_cast<char*>(&v), sizeof(T));
    if (!f) throw Error(MG_ERR_ARG, "truncated file: " + file.string());
    return v;
  }

  std::map<Path, size_t> path_to_index_;
  std::map<size_t, Path> index_to_path_;
  std::vector<Lab> labs_;
  std::vector<float> sims_;
  size_t built_n_ = 0;
};

// ---- adjacency.rs ------------------------------------------------------------------------
struct GridPosition {  // adjacency.rs:5-46
  size_t x = 0, y = 0;
  GridPosition() = default;
  GridPosition(size_t x_, size_t y_) : x(x_), y(y_) {}
  bool operator==(const GridPosition& o) const { return x == o.x && y == o.y; }
  bool operator!=(const GridPosition& o) const { return !(*this == o); }
  // Up, down, left, right -- the order the penalty sums in.
  std::vector<GridPosition> get_adjacent_positions(size_t grid_width, size_t grid_height) const {
    std::vector<GridPosition> v;
    if (y > 0) v.emplace_back(x, y - 1);
    if (y + 1 < grid_height) v.emplace_back(x, y + 1);
    if (x > 0) v.emplace_back(x - 1, y);
    if (x + 1 < grid_width) v.emplace_back(x + 1, y);
    return v;
  }
};

class AdjacencyPenaltyCalculator {
 public:
  AdjacencyPenaltyCalculator(const SimilarityDatabase& db, float penalty_weight, Context& ctx = default_context())
      : db_(&db), weight_(penalty_weight), ctx_(&ctx) {}

  // adjacency.rs:63-88: weight * sum over placed neighbours of 1/(sim+1); a
  // neighbour or candidate unknown to the database contributes nothing.
  float calculate_penalty(const Path& candidate, GridPosition pos, const Grid& grid, size_t grid_width,
                          size_t grid_height) const {
    require_built();
    auto ci = db_->index_of(candidate);
    if (!ci || grid_width == 0 || grid_height == 0) return 0.0f;
    std::vector<int32_t> g = indices(grid, grid_width, grid_height, false);
    const int32_t cxy[3] = {(int32_t)*ci, (int32_t)pos.x, (int32_t)pos.y};
    float out = 0.0f;
    const std::vector<float> lab = db_->flat_lab();
    detail::check(mg_penalty_batch(ctx_->get(), lab.data(), (int)db_->len(), g.data(), (int)grid_width,
                                   (int)grid_height, weight_, cxy, 1, &out));
    return out;
  }

  // adjacency.rs:91-130: unweighted sum over right and down pairs.
  float calculate_total_cost(const Grid& grid) const {
    require_built();
    if (grid.empty() || grid[0].empty()) return 0.0f;
    const size_t gw = grid[0].size(), gh = grid.size();
    std::vector<int32_t> g = indices(grid, gw, gh, false);
    float out = 0.0f;
    const std::vector<float> lab = db_->flat_lab();
    detail::check(mg_total_cost(ctx_->get(), lab.data(), (int)db_->len(), g.data(), (int)gw, (int)gh, &out));
    return out;
  }

  // adjacency.rs:133-214
  float calculate_swap_delta(const Grid& grid, GridPosition a, GridPosition b) const {
    require_built();
    if (grid.empty() || grid[0].empty()) return 0.0f;
    const size_t gw = grid[0].size(), gh = grid.size();
    std::vector<int32_t> g = indices(grid, gw, gh, false);
    const int32_t pairs[4] = {(int32_t)a.x, (int32_t)a.y, (int32_t)b.x, (int32_t)b.y};
    float out = 0.0f;
    const std::vector<float> lab = db_->flat_lab();
    detail::check(mg_swap_delta_batch(ctx_->get(), lab.data(), (int)db_->len(), g.data(), (int)gw, (int)gh, pairs, 1,
                                      &out));
    return out;
  }

  void require_built() const {
    if (!db_->built()) throw Error(MG_ERR_STATE, "build_similarities has not run over every tile");
  }
  const SimilarityDatabase& database() const { return *db_; }
  float weight() const { return weight_; }
  Context& context() const { return *ctx_; }

  // Row-major palette indices, -1 for an empty cell (and, unless `strict`, for
  // a tile the database does not know, which the crate's lookups skip too).
  std::vector<int32_t> indices(const Grid& grid, size_t gw, size_t gh, bool strict) const {
    std::vector<int32_t> g(gw * gh, -1);
    for (size_t y = 0; y < gh; ++y) {
      if (grid[y].size() != gw) throw Error(MG_ERR_ARG, "ragged grid");
      for (size_t x = 0; x < gw; ++x) {
        const auto& cell = grid[y][x];
        if (!cell) continue;
        auto i = db_->index_of(*cell);
        if (i) g[y * gw + x] = (int32_t)*i;
        else if (strict) throw Error(MG_ERR_ARG, "tile not in the similarity database: " + cell->string());
      }
    }
    return g;
  }

 private:
  const SimilarityDatabase* db_;
  float weight_;
  Context* ctx_;
};

// ---- optimizer.rs ---------------------------------------------------------------------------
struct OptimizationConfig {  // optimizer.rs:7-27 (+ seeded stream and chains)
  size_t max_iterations = 1000;
  float initial_temperature = 100.0f;
  float temperature_decay = 0.99995f;
  size_t report_interval = 100;  // kept for the crate's field set; nothing is printed
  uint64_t seed = 0;
  uint32_t stream = 0;
  int chains = 1;  // independent chains; the grid takes the lowest final cost
};

struct OptimizationResult {  // optimizer.rs:203-221
  float initial_cost = 0.0f, final_cost = 0.0f, best_cost = 0.0f;
  size_t improved_count = 0, accepted_count = 0, iterations = 0;
  float improvement_percentage() const {
    mg_sa_result r{};
    r.initial_cost = initial_cost;
    r.final_cost = final_cost;
    return mg_improvement_percentage(&r);
  }
};

class MosaicOptimizer {
 public:
  MosaicOptimizer(const AdjacencyPenaltyCalculator& calc, OptimizationConfig cfg) : calc_(&calc), cfg_(cfg) {}

  // optimizer.rs:41-129
  OptimizationResult optimize(Grid& grid) const { return run(grid, cfg_.max_iterations, false); }
  // optimizer.rs:132-198
  OptimizationResult optimize_greedy(Grid& grid, size_t max_iterations) const { return run(grid, max_iterations, true); }

 private:
  OptimizationResult run(Grid& grid, size_t iters, bool greedy) const {
    if (grid.empty()) return {};
    const size_t gw = grid[0].size(), gh = grid.size();
    const SimilarityDatabase& db = calc_->database();
    calc_->require_built();
    std::vector<int32_t> g = calc_->indices(grid, gw, gh, true);
    mg_sa_config c;
    mg_sa_config_default(&c);
    c.max_iterations = (int64_t)iters;
    c.initial_temperature = cfg_.initial_temperature;
    c.temperature_decay = cfg_.temperature_decay;
    c.chains = cfg_.chains;
    c.seed = cfg_.seed;
    c.stream = cfg_.stream;
    c.greedy_only = greedy ? 1 : 0;
    mg_sa_result best{};
    const std::vector<float> lab = db.flat_lab();
    detail::check(mg_optimize(calc_->context().get(), lab.data(), (int)db.len(), g.data(), (int)gw, (int)gh, &c,
                              &best, nullptr, nullptr));
    for (size_t y = 0; y < gh; ++y)
      for (size_t x = 0; x < gw; ++x) {
        const int32_t i = g[y * gw + x];
        grid[y][x] = i >= 0 ? std::optional<Path>(db.path_of((size_t)i)) : std::nullopt;
      }
    OptimizationResult r;
    r.initial_cost = best.initial_cost;
    r.final_cost = best.final_cost;
    r.best_cost = best.best_cost;
    r.improved_count = (size_t)best.improved_count;
    r.accepted_count = (size_t)best.accepted_count;
    r.iterations = (size_t)best.iterations;
    return r;
  }

  const AdjacencyPenaltyCalculator* calc_;
  OptimizationConfig cfg_;
};

// ---- color_adjustment.rs -----------------------------------------------------------------------
struct ColorAdjustment {  // color_adjustment.rs:6-26
  float brightness = 0.0f, contrast = 1.0f, hue_shift = 0.0f, saturation = 1.0f;

  // color_adjustment.rs:30-37 (ColorAdjustment::new, clamping each field)
  static ColorAdjustment create(float brightness, float contrast, float hue_shift, float saturation) {
    const mg_color_adjustment a = mg_color_adjustment_new(brightness, contrast, hue_shift, saturation);
    return {a.brightness, a.contrast, a.hue_shift, a.saturation};
  }
  mg_color_adjustment raw() const { return {brightness, contrast, hue_shift, saturation}; }

  // color_adjustment.rs:53-89
  Rgb adjust_pixel(Rgb px, Context& ctx = default_context()) const {
    const uint8_t in[3] = {px.r, px.g, px.b};
    uint8_t out[3];
    const mg_color_adjustment a = raw();
    detail::check(mg_apply_adjustment(ctx.get(), &a, in, 1, 1, 3, out));
    return {out[0], out[1], out[2]};
  }
  // color_adjustment.rs:40-51
  RgbImage apply_to_image(const RgbImageView& img, Context& ctx = default_context()) const {
    RgbImage out;
    out.width = img.width;
    out.height = img.height;
    out.pixels.resize((size_t)img.width * img.height * 3);
    const mg_color_adjustment a = raw();
    detail::check(mg_apply_adjustment(ctx.get(), &a, img.data, img.width, img.height, img.row_bytes(),
                                      out.pixels.data()));
    return out;
  }
};

// color_adjustment.rs:99-154
inline ColorAdjustment calculate_optimal_adjustment(Rgb tile_avg, Rgb target_avg, float strength,
                                                    Context& ctx = default_context()) {
  const uint8_t t[3] = {tile_avg.r, tile_avg.g, tile_avg.b}, g[3] = {target_avg.r, target_avg.g, target_avg.b};
  mg_color_adjustment a;
  detail::check(mg_optimal_adjustment_batch(ctx.get(), t, g, 1, strength, &a));
  return {a.brightness, a.contrast, a.hue_shift, a.saturation};
}

// ---- the generator (main.rs) --------------------------------------------------------------------
// The CLI options of main.rs:21-88 that reach the path.
struct MosaicOptions {
  int grid_w = 50, grid_h = 28;
  int max_materials = 500;
  float aspect_tolerance = 0.1f;
  int max_usage_per_image = 3;
  float adjacency_penalty_weight = 0.3f;
  bool enable_optimization = true;
  int64_t optimization_iterations = 1000;
  float color_adjustment_strength = 0.3f;
  int tile_w = 0, tile_h = 0;  // 0 -> cell size
  int chains = 1;
  uint64_t seed = 0;
  uint32_t stream = 0;
  bool build_similarity = true;
};

struct MosaicOutput {
  Grid grid;  // grid[y][x]: the material's path, or empty
  RgbImage image;
  int palette_size = 0, n_resets = 0;
  OptimizationResult optimization;
};

// main.rs:105-164 (palette ingestion) + main.rs:477-685 (generate_mosaic) from
// decoded images; materials[i] is named paths[i].  When no material survives
// load_tiles every cell stays empty (main.rs:342-345 returns None per cell).
inline MosaicOutput generate_mosaic(const RgbImageView& target, const std::vector<RgbImageView>& materials,
                                                   const std::vector<Path>& paths, const MosaicOptions& o,
                                                   const uint8_t* thumbnails = nullptr,
                                                   Context& ctx = default_context()) {
  if (materials.size() != paths.size()) throw Error(MG_ERR_ARG, "one path per material");
  const int n = (int)materials.size();
  std::vector<const uint8_t*> ptrs(n);
  std::vector<int> w(n), h(n);
  std::vector<int64_t> s(n);
  for (int i = 0; i < n; ++i) {
    ptrs[i] = materials[i].data;
    w[i] = materials[i].width;
    h[i] = materials[i].height;
    s[i] = materials[i].row_bytes();
  }
  mg_request r;
  mg_request_default(&r);
  r.target = target.data;
  r.target_w = target.width;
  r.target_h = target.height;
  r.target_stride = target.row_bytes();
  r.n_materials = n;
  r.materials = ptrs.data();
  r.material_w = w.data();
  r.material_h = h.data();
  r.material_stride = s.data();
  r.thumbnails = thumbnails;
  r.tile_w = o.tile_w;
  r.tile_h = o.tile_h;
  r.grid_w = o.grid_w;
  r.grid_h = o.grid_h;
  r.max_materials = o.max_materials;
  r.aspect_tolerance = o.aspect_tolerance;
  r.max_usage_per_image = o.max_usage_per_image;
  r.adjacency_penalty_weight = o.adjacency_penalty_weight;
  r.color_adjustment_strength = o.color_adjustment_strength;
  r.enable_optimization = o.enable_optimization ? 1 : 0;
  r.optimization_iterations = o.optimization_iterations;
  r.chains = o.chains;
  r.seed = o.seed;
  r.stream = o.stream;
  r.build_similarity = o.build_similarity ? 1 : 0;
  const int tw = o.tile_w ? o.tile_w : (o.grid_w > 0 ? target.width / o.grid_w : 0);
  const int th = o.tile_h ? o.tile_h : (o.grid_h > 0 ? target.height / o.grid_h : 0);
  std::vector<int32_t> grid((size_t)std::max(o.grid_w, 0) * std::max(o.grid_h, 0));
  MosaicOutput out;
  out.image.width = o.grid_w * tw;
  out.image.height = o.grid_h * th;
  out.image.pixels.resize((size_t)out.image.width * out.image.height * 3);
  mg_result res{};
  res.grid = grid.data();
  res.image = out.image.pixels.data();
  detail::check(mg_generate(ctx.get(), &r, &res));
  out.palette_size = res.palette_size;
  out.n_resets = res.n_resets;
  out.optimization.initial_cost = res.initial_cost;
  out.optimization.final_cost = res.final_cost;
  out.optimization.best_cost = res.best_cost;
  out.optimization.accepted_count = (size_t)res.accepted_count;
  out.optimization.improved_count = (size_t)res.improved_count;
  out.optimization.iterations = o.enable_optimization ? (size_t)o.optimization_iterations : 0;
  out.grid.assign(o.grid_h, std::vector<std::optional<Path>>(o.grid_w));
  for (int y = 0; y < o.grid_h; ++y)
    for (int x = 0; x < o.grid_w; ++x) {
      const int32_t i = grid[(size_t)y * o.grid_w + x];
      if (i >= 0) out.grid[y][x] = paths[(size_t)i];
    }
  return out;
}

// main.rs:105-164 + 477-685 from files: the target (PNG or JPEG), the
// material folder (read_material_files on up to `threads` host threads) and,
// when output_path is not empty, the mosaic saved there after creating its
// parent folders (main.rs:667-672; the format by extension as the crate picks
// it: save_image writes .png and .jpg / .jpeg, any other fails with
// MG_ERR_ARG before any work).  Files skipped while reading are listed in
// *skipped.
inline MosaicOutput generate_mosaic_files(const Path& target_path, const Path& material_dir, const Path& output_path,
                                          const MosaicOptions& o, int threads = 0,
                                          std::vector<std::pair<Path, std::string>>* skipped = nullptr,
                                          Context& ctx = default_context()) {
  if (!output_path.empty()) {
    std::string ext = output_path.extension().string();
    for (char& c : ext) c = (char)std::tolower((unsigned char)c);
    if (ext != ".png" && ext != ".jpg" && ext != ".jpeg")
      throw Error(MG_ERR_ARG, "only PNG and JPEG output is written: " + output_path.string());
  }
  const RgbImage target = open_image(target_path);
  const MaterialFiles m = read_material_files(material_dir, threads);
  if (skipped) *skipped = m.errors;
  MosaicOutput out = generate_mosaic(target.view(), m.views(), m.paths, o, nullptr, ctx);
  if (!output_path.empty()) {
    if (output_path.has_parent_path()) std::filesystem::create_directories(output_path.parent_path());
    save_image(out.image.view(), output_path, threads);
  }
  return out;
}

// ---- resident palette, batches, serving (no counterpart in the crate) -------------------------------
class Palette {
 public:
  Palette(const std::vector<RgbImageView>& materials, const uint8_t* thumbnails, int tile_w, int tile_h,
          float target_aspect, float aspect_tolerance = 0.1f, int max_materials = 0, bool build_similarity = true,
          Context& ctx = default_context()) {
    const int n = (int)materials.size();
    std::vector<const uint8_t*> ptrs(n);
    std::vector<int> w(n), h(n);
    std::vector<int64_t> s(n);
    for (int i = 0; i < n; ++i) {
      ptrs[i] = materials[i].data;
      w[i] = materials[i].width;
      h[i] = materials[i].height;
      s[i] = materials[i].row_bytes();
    }
    mg_palette_desc d;
    mg_palette_desc_default(&d);
    d.n_materials = n;
    d.materials = ptrs.data();
    d.material_w = w.data();
    d.material_h = h.data();
    d.material_stride = s.data();
    d.thumbnails = thumbnails;
    d.tile_w = tile_w;
    d.tile_h = tile_h;
    d.target_aspect = target_aspect;
    d.aspect_tolerance = aspect_tolerance;
    d.max_materials = max_materials ? max_materials : n;
    d.build_similarity = build_similarity ? 1 : 0;
    detail::check(mg_palette_create(ctx.get(), &d, &h_));
  }
  ~Palette() {
    if (h_) mg_palette_destroy(h_);
  }
  Palette(const Palette&) = delete;
  Palette& operator=(const Palette&) = delete;
  mg_palette* get() const { return h_; }
  int size() const { return mg_palette_size(h_); }

 private:
  mg_palette* h_ = nullptr;
};

class Server {
 public:
  Server(Palette& pal, int slots = 3, int max_batch = 64, int64_t memory_budget_bytes = 120ll << 30,
         Context& ctx = default_context()) {
    mg_server_config c;
    mg_server_config_default(&c);
    c.slots = slots;
    c.max_batch = max_batch;
    c.memory_budget_bytes = memory_budget_bytes;
    detail::check(mg_server_create(ctx.get(), pal.get(), &c, &h_));
  }
  ~Server() {
    if (h_) mg_server_destroy(h_);
  }
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;
  // The target and outputs must stay valid until the request completes.
  uint64_t submit(const mg_mosaic& m, int32_t* grid_out, uint8_t* image_out) {
    uint64_t t = 0;
    detail::check(mg_server_submit(h_, &m, grid_out, image_out, &t));
    return t;
  }
  // Status (MG_OK or MG_ERR_BUDGET), the result summary and the latency in ms.
  int wait(uint64_t ticket, mg_result* res, double* latency_ms) { return mg_server_wait(h_, ticket, res, latency_ms); }
  mg_server_stats stats() const {
    mg_server_stats s{};
    detail::check(mg_server_get_stats(h_, &s));
    return s;
  }

 private:
  mg_server* h_ = nullptr;
};

}  // namespace mosaic

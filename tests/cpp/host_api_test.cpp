// host_api_test.cpp -- the crate's own unit tests, restated against the C++
// mirror (mosaic-art-rust_gb300/host/mosaic.hpp) over libmosaic_gpu.so.
//
//   host_api_test --cpu    host-side parts (UsageTracker, GridPosition, the
//                          similarity database file format, clamps, ...), and
//                          that a missing GPU surfaces as mosaic::Error
//   host_api_test --gpu    everything, on device 0
//
// Each block names the reference test it restates (file:line in the crate).
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "mosaic.hpp"

using namespace mosaic;

static int g_failed = 0, g_checked = 0;
#define CHECK(cond)                                                          \
  do {                                                                       \
    ++g_checked;                                                             \
    if (!(cond)) {                                                           \
      ++g_failed;                                                            \
      std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
    }                                                                        \
  } while (0)

static Path tmp_file(const char* name) {
  return std::filesystem::temp_directory_path() / (std::string("mg_host_api_") + std::to_string(::getpid()) + name);
}

// ---------------------------------------------------------------- host only
static void usage_tracker_tests() {  // lib.rs:242-306
  {
    UsageTracker t(3);
    CHECK(t.can_use_image("test.png"));
    CHECK(t.get_usage_count("test.png") == 0);
  }
  {
    UsageTracker t(2);
    CHECK(t.can_use_image("test.png"));
    t.use_image("test.png");
    CHECK(t.get_usage_count("test.png") == 1);
    CHECK(t.can_use_image("test.png"));
    t.use_image("test.png");
    CHECK(t.get_usage_count("test.png") == 2);
    CHECK(!t.can_use_image("test.png"));
  }
  {
    UsageTracker t(1);
    t.use_image("image1.png");
    CHECK(!t.can_use_image("image1.png"));
    CHECK(t.can_use_image("image2.png"));
    t.use_image("image2.png");
    CHECK(!t.can_use_image("image2.png"));
  }
  {
    UsageTracker t(1);
    t.use_image("test.png");
    CHECK(!t.can_use_image("test.png"));
    t.reset();
    CHECK(t.can_use_image("test.png"));
    CHECK(t.get_usage_count("test.png") == 0);
  }
  {
    UsageTracker t(0);
    CHECK(!t.can_use_image("test.png"));
  }
}

static void aspect_tests() {  // lib.rs:160-209
  CHECK(MosaicGeneratorImpl::is_aspect_ratio_match(16.0f / 9.0f, 16.0f / 9.0f, 0.1f));
  CHECK(MosaicGeneratorImpl::is_aspect_ratio_match(1.8f, 16.0f / 9.0f, 0.1f));
  CHECK(!MosaicGeneratorImpl::is_aspect_ratio_match(4.0f / 3.0f, 16.0f / 9.0f, 0.1f));
  CHECK(!MosaicGeneratorImpl::is_aspect_ratio_match(16.0f / 9.0f, 9.0f / 16.0f, 0.1f));
}

static bool contains(const std::vector<GridPosition>& v, GridPosition p) {
  for (auto& q : v)
    if (q == p) return true;
  return false;
}

static void grid_position_tests() {  // adjacency.rs:224-244
  auto adj = GridPosition(1, 1).get_adjacent_positions(3, 3);
  CHECK(adj.size() == 4);
  CHECK(contains(adj, {1, 0}) && contains(adj, {1, 2}) && contains(adj, {0, 1}) && contains(adj, {2, 1}));
  // up, down, left, right is the order the penalty sums in
  CHECK(adj[0] == GridPosition(1, 0) && adj[1] == GridPosition(1, 2) && adj[2] == GridPosition(0, 1) &&
        adj[3] == GridPosition(2, 1));
  auto corner = GridPosition(0, 0).get_adjacent_positions(3, 3);
  CHECK(corner.size() == 2 && contains(corner, {1, 0}) && contains(corner, {0, 1}));
}

static void lab_distance_tests() {  // similarity.rs:207-218
  Lab a{50, 0, 0}, b{50, 0, 0}, c{60, 10, 10};
  CHECK(calculate_lab_distance(a, b) == 0.0f);
  CHECK(calculate_lab_distance(a, c) > 0.0f);
  CHECK(calculate_lab_distance(a, c) == std::sqrt(300.0f));
}

static void similarity_host_tests() {
  {  // similarity.rs:235-253
    SimilarityDatabase db;
    db.add_tile("test.png", {50, 25, -15});
    auto l = db.get_lab_color("test.png");
    CHECK(l && l->l == 50.0f && l->a == 25.0f && l->b == -15.0f);
    CHECK(!db.get_lab_color("nonexistent.png"));
  }
  {  // similarity.rs:308-319
    SimilarityDatabase db;
    CHECK(!db.get_similarity("tile1.png", "tile2.png"));
    CHECK(!db.get_lab_color("tile1.png"));
  }
  {  // similarity.rs:281-297 (an unbuilt database round-trips without a GPU)
    SimilarityDatabase none = SimilarityDatabase::load_or_new("nonexistent_db.bin");
    CHECK(none.len() == 0);
    SimilarityDatabase db;
    db.add_tile("test.png", {50, 0, 0});
    const Path f = tmp_file("_one.bin");
    db.save_to_file(f);
    SimilarityDatabase back = SimilarityDatabase::load_or_new(f);
    CHECK(back.len() == 1);
    CHECK(back.get_lab_color("test.png") && back.get_lab_color("test.png")->l == 50.0f);
    std::filesystem::remove(f);
  }
  {  // similarity.rs:299-306
    const Path f = tmp_file("_bad.bin");
    {
      std::ofstream o(f);
      o << "invalid json";
    }
    bool threw = false;
    try {
      SimilarityDatabase::load_from_file(f);
    } catch (const Error&) {
      threw = true;
    }
    CHECK(threw);
    std::filesystem::remove(f);
  }
}

// The crate's own database file (serde_json::to_string_pretty of
// similarity.rs:31-41, save_to_file :112-116) loads unchanged, is written back
// in the same layout, and defects in it are errors.
static void similarity_json_tests() {
  const Path f = tmp_file("_crate.json"), f2 = tmp_file("_back.json"), f3 = tmp_file("_back.bin");
  const std::string q = "tiles/a \"q\" \xc3\xbc.png";  // a quote and a non-ASCII letter in the path
  {
    std::ofstream o(f);
    o << R"({
  "path_to_index": {
    "tiles/b.png": 1,
    "tiles/a \"q\" \u00fc.png": 0,
    "tiles/c.png": 2
  },
  "index_to_path": {
    "1": "tiles/b.png",
    "0": "tiles/a \"q\" \u00fc.png",
    "2": "tiles/c.png"
  },
  "lab_colors": [
    {
      "l": 50.0,
      "a": 25.0,
      "b": -15.0
    },
    {
      "l": 53.23288,
      "a": 80.10931,
      "b": 67.22006
    },
    {
      "l": 0.0,
      "a": -0.0,
      "b": 1e-7
    }
  ],
  "similarities": [
    1.5,
    2.25,
    0.3
  ]
})";
  }
  SimilarityDatabase db = SimilarityDatabase::load_or_new(f);
  CHECK(db.len() == 3 && db.built());
  CHECK(db.index_of(q) && *db.index_of(q) == 0 && db.path_of(2) == Path("tiles/c.png"));
  CHECK(db.get_lab_color("tiles/b.png") && db.get_lab_color("tiles/b.png")->l == 53.23288f &&
        db.get_lab_color("tiles/b.png")->b == 67.22006f && db.get_lab_color("tiles/c.png")->b == 1e-7f);
  CHECK(db.get_similarity(q, "tiles/b.png") == 1.5f && db.get_similarity("tiles/c.png", q) == 2.25f &&
        db.get_similarity("tiles/b.png", "tiles/c.png") == 0.3f);
  db.save_json(f2);
  SimilarityDatabase back = SimilarityDatabase::load_from_file(f2);
  db.save_to_file(f3);
  SimilarityDatabase bin = SimilarityDatabase::load_from_file(f3);
  for (const SimilarityDatabase* d : {&back, &bin}) {
    CHECK(d->len() == 3 && d->built() && d->similarities() == db.similarities() && d->flat_lab() == db.flat_lab());
    for (size_t i = 0; i < 3; ++i) CHECK(d->path_of(i) == db.path_of(i));
  }
  {
    std::ifstream in(f2);
    const std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    CHECK(text.find("\"path_to_index\": {") != std::string::npos && text.find("\"0\": \"tiles/a \\\"q\\\"") != std::string::npos);
  }
  {  // an empty database written by the crate
    std::ofstream o(f);
    o << "{\n  \"path_to_index\": {},\n  \"index_to_path\": {},\n  \"lab_colors\": [],\n  \"similarities\": []\n}";
  }
  SimilarityDatabase empty = SimilarityDatabase::load_from_file(f);
  CHECK(empty.len() == 0 && !empty.built());
  empty.save_json(f2);
  CHECK(SimilarityDatabase::load_from_file(f2).len() == 0);
  // defects: each throws mosaic::Error (load_or_new then starts a new database)
  const char* bad[] = {
      "{\"path_to_index\": {}, \"index_to_path\": {\"0\": \"a.png\"}, \"lab_colors\": [], \"similarities\": []}",
      "{\"index_to_path\": {\"0\": \"a.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2}], \"similarities\": []}",
      "{\"index_to_path\": {\"0\": \"a.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": \"x\"}], \"similarities\": []}",
      "{\"index_to_path\": {\"0\": \"a\\q.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": 3}], \"similarities\": []}",
      "{\"index_to_path\": {\"-1\": \"a.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": 3}], \"similarities\": []}",
      "{\"index_to_path\": {\"0\": \"a.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": 3}], \"similarities\": [1,]}",
      "{\"index_to_path\": {\"0\": \"a.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": 3}], \"similarities\": []",
      "{\"index_to_path\": {\"0\": \"\\ud800.png\"}, \"lab_colors\": [{\"l\": 1, \"a\": 2, \"b\": 3}], \"similarities\": []}",
      "{\"lab_colors\": [], \"similarities\": []}",
      "  {"};
  for (const char* t : bad) {
    {
      std::ofstream o(f);
      o << t;
    }
    bool threw = false;
    try {
      SimilarityDatabase::load_from_file(f);
    } catch (const Error&) {
      threw = true;
    }
    CHECK(threw);
    CHECK(SimilarityDatabase::load_or_new(f).len() == 0);
  }
  for (const Path& p : {f, f2, f3}) std::filesystem::remove(p);
}

static void color_host_tests() {  // color_adjustment.rs:160-178
  ColorAdjustment d;
  CHECK(d.brightness == 0.0f && d.contrast == 1.0f && d.hue_shift == 0.0f && d.saturation == 1.0f);
  ColorAdjustment c = ColorAdjustment::create(2.0f, 3.0f, 200.0f, -1.0f);
  CHECK(c.brightness == 1.0f && c.contrast == 2.0f && c.hue_shift == 180.0f && c.saturation == 0.0f);
}

static void result_tests() {  // optimizer.rs:280-292, 550-587
  OptimizationResult r;
  r.initial_cost = 100.0f;
  r.final_cost = 75.0f;
  CHECK(r.improvement_percentage() == 25.0f);
  OptimizationResult z;
  CHECK(z.improvement_percentage() == 0.0f);
  OptimizationConfig cfg;  // optimizer.rs:621-629
  CHECK(cfg.max_iterations == 1000 && cfg.initial_temperature == 100.0f && cfg.temperature_decay == 0.99995f &&
        cfg.report_interval == 100);
}

// ---------------------------------------------------------------- device
static std::vector<uint8_t> solid(int w, int h, uint8_t r, uint8_t g, uint8_t b) {
  std::vector<uint8_t> v((size_t)w * h * 3);
  for (size_t i = 0; i < v.size(); i += 3) {
    v[i] = r;
    v[i + 1] = g;
    v[i + 2] = b;
  }
  return v;
}

static void average_lab_tests() {  // lib.rs:133-158
  auto red = solid(10, 10, 255, 0, 0);
  Lab l = MosaicGeneratorImpl::calculate_average_lab({red.data(), 10, 10, 0});
  CHECK(std::fabs(l.l - 53.24f) < 1.0f && std::fabs(l.a - 80.09f) < 1.0f && std::fabs(l.b - 67.20f) < 1.0f);
  auto grey = solid(10, 10, 128, 128, 128);
  Lab g = MosaicGeneratorImpl::calculate_average_lab({grey.data(), 10, 10, 0});
  CHECK(std::fabs(g.l - 53.59f) < 1.0f && std::fabs(g.a) < 1.0f && std::fabs(g.b) < 1.0f);
}

static SimilarityDatabase three_tiles() {
  SimilarityDatabase db;
  db.add_tile("tile1.png", {50, 0, 0});
  db.add_tile("tile2.png", {60, 10, 10});
  db.add_tile("tile3.png", {40, -10, -10});
  db.build_similarities();
  return db;
}

static void similarity_device_tests() {
  {  // similarity.rs:186-204, 336-361
    SimilarityDatabase db = three_tiles();
    auto s12 = db.get_similarity("tile1.png", "tile2.png"), s21 = db.get_similarity("tile2.png", "tile1.png");
    auto s13 = db.get_similarity("tile1.png", "tile3.png"), s23 = db.get_similarity("tile2.png", "tile3.png");
    CHECK(s12 && s21 && s13 && s23);
    CHECK(*s12 == *s21 && *s12 > 0 && *s13 > 0 && *s23 > 0);
    CHECK(db.get_similarity("tile1.png", "tile1.png") == std::optional<float>(0.0f));
    // the stored value is calculate_lab_distance of the two colours, bit for bit
    CHECK(*s12 == calculate_lab_distance({50, 0, 0}, {60, 10, 10}));
    CHECK(*s23 == calculate_lab_distance({60, 10, 10}, {40, -10, -10}));
  }
  {  // similarity.rs:321-334
    SimilarityDatabase db;
    db.add_tile("tile1.png", {50, 0, 0});
    db.build_similarities();
    CHECK(db.get_similarity("tile1.png", "tile1.png") == std::optional<float>(0.0f));
    CHECK(!db.get_similarity("tile1.png", "nonexistent.png"));
  }
  {  // similarity.rs:255-279: save, load, similarities preserved bit for bit
    SimilarityDatabase db = three_tiles();
    const Path f = tmp_file("_three.bin");
    db.save_to_file(f);
    SimilarityDatabase back = SimilarityDatabase::load_from_file(f);
    CHECK(back.len() == 3 && back.built());
    CHECK(back.similarities() == db.similarities());
    CHECK(back.get_similarity("tile1.png", "tile2.png") == db.get_similarity("tile1.png", "tile2.png"));
    std::filesystem::remove(f);
  }
}

static Grid grid_of(size_t w, size_t h) { return Grid(h, std::vector<std::optional<Path>>(w)); }

static void adjacency_device_tests() {
  {  // adjacency.rs:246-272
    SimilarityDatabase db = three_tiles();
    AdjacencyPenaltyCalculator calc(db, 1.0f);
    Grid g = grid_of(3, 3);
    g[0][0] = Path("tile1.png");
    g[0][1] = Path("tile2.png");
    const float p = calc.calculate_penalty("tile3.png", GridPosition(1, 0), g, 3, 3);
    CHECK(p > 0.0f);
    // only the left neighbour (tile1) is placed around (1, 0)
    CHECK(p == 1.0f / (calculate_lab_distance({40, -10, -10}, {50, 0, 0}) + 1.0f));
    CHECK(calc.calculate_penalty("unknown.png", GridPosition(1, 0), g, 3, 3) == 0.0f);
  }
  {  // adjacency.rs:274-290
    SimilarityDatabase db;
    db.add_tile("tile1.png", {50, 0, 0});
    db.add_tile("tile2.png", {50, 0, 0});
    db.build_similarities();
    AdjacencyPenaltyCalculator calc(db, 1.0f);
    Grid g = grid_of(2, 2);
    g[0][0] = Path("tile1.png");
    g[0][1] = Path("tile2.png");
    CHECK(calc.calculate_total_cost(g) > 0.5f);
    CHECK(calc.calculate_total_cost(g) == 1.0f);
  }
  {  // a swap of two cells with the same neighbourhood changes nothing
    SimilarityDatabase db = three_tiles();
    AdjacencyPenaltyCalculator calc(db, 1.0f);
    Grid g = grid_of(2, 1);
    g[0][0] = Path("tile1.png");
    g[0][1] = Path("tile2.png");
    CHECK(calc.calculate_swap_delta(g, GridPosition(0, 0), GridPosition(1, 0)) == 0.0f);
  }
  {  // unbuilt database: an error, not a silent zero
    SimilarityDatabase db;
    db.add_tile("tile1.png", {50, 0, 0});
    AdjacencyPenaltyCalculator calc(db, 1.0f);
    Grid g = grid_of(1, 1);
    g[0][0] = Path("tile1.png");
    bool threw = false;
    try {
      calc.calculate_total_cost(g);
    } catch (const Error& e) {
      threw = e.code() == MG_ERR_STATE;
    }
    CHECK(threw);
  }
}

static void optimizer_device_tests() {
  SimilarityDatabase db;
  db.add_tile("tile1.png", {50, 0, 0});
  db.add_tile("tile2.png", {60, 10, 10});
  db.add_tile("tile3.png", {40, -10, -10});
  db.add_tile("tile4.png", {55, 5, 5});
  db.build_similarities();
  auto test_grid = [] {
    Grid g = grid_of(2, 2);
    g[0][0] = Path("tile1.png");
    g[0][1] = Path("tile2.png");
    g[1][0] = Path("tile3.png");
    g[1][1] = Path("tile4.png");
    return g;
  };
  AdjacencyPenaltyCalculator calc(db, 1.0f);
  {  // optimizer.rs:247-264
    OptimizationConfig cfg;
    cfg.max_iterations = 10;
    Grid g = test_grid();
    OptimizationResult r = MosaicOptimizer(calc, cfg).optimize(g);
    CHECK(r.iterations == 10 && r.final_cost >= 0.0f);
    // the final grid is a permutation of the start
    std::vector<std::string> seen;
    for (auto& row : g)
      for (auto& c : row) seen.push_back(c ? c->string() : "");
    std::sort(seen.begin(), seen.end());
    CHECK((seen == std::vector<std::string>{"tile1.png", "tile2.png", "tile3.png", "tile4.png"}));
    CHECK(std::fabs(calc.calculate_total_cost(g) - r.final_cost) <= 1e-5f * std::max(1.0f, r.final_cost));
  }
  {  // optimizer.rs:266-278
    Grid g = test_grid();
    OptimizationResult r = MosaicOptimizer(calc, OptimizationConfig()).optimize_greedy(g, 10);
    CHECK(r.final_cost <= r.initial_cost && r.improved_count == r.accepted_count);
  }
  {  // optimizer.rs:294-307 (empty grid, empty database)
    SimilarityDatabase empty;
    AdjacencyPenaltyCalculator c0(empty, 1.0f);
    Grid g;
    OptimizationResult r = MosaicOptimizer(c0, OptimizationConfig()).optimize(g);
    CHECK(r.initial_cost == 0.0f && r.final_cost == 0.0f && r.improved_count == 0);
  }
  {  // optimizer.rs:309-331
    SimilarityDatabase one;
    one.add_tile("single.png", {50, 0, 0});
    one.build_similarities();
    AdjacencyPenaltyCalculator c1(one, 1.0f);
    Grid g = grid_of(1, 1);
    g[0][0] = Path("single.png");
    OptimizationConfig cfg;
    cfg.max_iterations = 100;
    OptimizationResult r = MosaicOptimizer(c1, cfg).optimize(g);
    CHECK(r.initial_cost == 0.0f && r.final_cost == 0.0f && r.improved_count == 0 && r.accepted_count == 0);
  }
  {  // optimizer.rs:333-358
    SimilarityDatabase two;
    two.add_tile("tile1.png", {50, 0, 0});
    two.add_tile("tile2.png", {60, 10, 10});
    two.build_similarities();
    AdjacencyPenaltyCalculator c2(two, 1.0f);
    Grid g = grid_of(3, 3);
    g[0][0] = Path("tile1.png");
    g[2][2] = Path("tile2.png");
    OptimizationConfig cfg;
    cfg.max_iterations = 50;
    OptimizationResult r = MosaicOptimizer(c2, cfg).optimize(g);
    CHECK(r.final_cost >= 0.0f && r.initial_cost == 0.0f);
  }
  {  // optimizer.rs:440-458
    OptimizationConfig cfg;
    cfg.max_iterations = 0;
    Grid g = test_grid();
    Grid before = g;
    OptimizationResult r = MosaicOptimizer(calc, cfg).optimize(g);
    CHECK(r.initial_cost == r.final_cost && r.iterations == 0 && g == before);
  }
  {  // a tile the database does not know cannot be optimised on the device
    Grid g = test_grid();
    g[1][1] = Path("stranger.png");
    bool threw = false;
    try {
      MosaicOptimizer(calc, OptimizationConfig()).optimize(g);
    } catch (const Error& e) {
      threw = e.code() == MG_ERR_ARG;
    }
    CHECK(threw);
  }
}

static void color_device_tests() {
  ColorAdjustment d;  // color_adjustment.rs:179-193
  for (Rgb px : {Rgb{128, 64, 192}, Rgb{0, 0, 0}, Rgb{255, 255, 255}, Rgb{10, 200, 30}}) {
    Rgb o = d.adjust_pixel(px);
    CHECK(std::abs(o.r - px.r) <= 1 && std::abs(o.g - px.g) <= 1 && std::abs(o.b - px.b) <= 1);
  }
  ColorAdjustment a = calculate_optimal_adjustment({128, 128, 128}, {128, 128, 128}, 1.0f);  // :221-231
  CHECK(std::fabs(a.brightness) < 0.01f && std::fabs(a.hue_shift) < 1.0f);
  ColorAdjustment up = ColorAdjustment::create(0.5f, 1.0f, 0.0f, 1.0f);  // :195-205
  Rgb o = up.adjust_pixel({100, 100, 100});
  CHECK(o.r > 100 && o.g > 100 && o.b > 100);
  auto img = solid(7, 5, 100, 150, 200);
  RgbImage out = up.apply_to_image({img.data(), 7, 5, 0});  // :321-353
  CHECK(out.width == 7 && out.height == 5 && out.pixels.size() == img.size());
  Rgb first{out.pixels[0], out.pixels[1], out.pixels[2]};
  Rgb single = up.adjust_pixel({100, 150, 200});
  CHECK(first.r == single.r && first.g == single.g && first.b == single.b);
}

static uint32_t lcg(uint32_t& s) { return s = s * 1664525u + 1013904223u; }

static void generate_tests() {
  // main.rs:1380-1424: output is grid_w*tile_w x grid_h*tile_h; every cell filled
  const int tw = 120, th = 90, gw = 12, gh = 9;
  std::vector<uint8_t> target((size_t)tw * th * 3);
  uint32_t s = 7;
  for (int y = 0; y < th; ++y)
    for (int x = 0; x < tw; ++x) {
      uint8_t* p = &target[((size_t)y * tw + x) * 3];
      p[0] = (uint8_t)(x * 2);
      p[1] = (uint8_t)(y * 2);
      p[2] = (uint8_t)(lcg(s) >> 24);
    }
  const int n = 40, side = 16;
  std::vector<std::vector<uint8_t>> mats(n);
  std::vector<RgbImageView> views;
  std::vector<Path> paths;
  for (int i = 0; i < n; ++i) {
    mats[i] = solid(side * 4 / 3, side, (uint8_t)(lcg(s) >> 24), (uint8_t)(lcg(s) >> 24), (uint8_t)(lcg(s) >> 24));
    views.push_back({mats[i].data(), side * 4 / 3, side, 0});
    paths.push_back("mat_" + std::to_string(i) + ".png");
  }
  MosaicOptions o;
  o.grid_w = gw;
  o.grid_h = gh;
  o.max_usage_per_image = 4;
  o.optimization_iterations = 500;
  o.tile_w = 8;
  o.tile_h = 6;
  o.seed = 99;
  MosaicOutput out = generate_mosaic({target.data(), tw, th, 0}, views, paths, o);
  CHECK(out.image.width == gw * 8 && out.image.height == gh * 6);
  CHECK(out.palette_size == n);
  bool filled = true;
  for (auto& row : out.grid)
    for (auto& c : row) filled = filled && c.has_value();
  CHECK(filled && (int)out.grid.size() == gh && (int)out.grid[0].size() == gw);
  MosaicOutput again = generate_mosaic({target.data(), tw, th, 0}, views, paths, o);
  CHECK(again.grid == out.grid && again.image.pixels == out.image.pixels);  // seeded: repeatable

  // main.rs:338-345: no tiles -> every cell stays empty
  MosaicOutput none = generate_mosaic({target.data(), tw, th, 0}, {}, {}, o);
  bool empty = true;
  for (auto& row : none.grid)
    for (auto& c : row) empty = empty && !c.has_value();
  CHECK(empty && none.palette_size == 0);
}

static void png_tests() {  // main.rs:1888-1912 (missing, corrupted files), 2219-2240 (save, then load)
  RgbImage red;  // create_test_image(100, 100, Rgb([255, 0, 0]))
  red.width = red.height = 100;
  red.pixels.resize(100 * 100 * 3);
  for (size_t i = 0; i < red.pixels.size(); i += 3) red.pixels[i] = 255;
  RgbImage noise;
  noise.width = 37;
  noise.height = 23;
  noise.pixels.resize(37 * 23 * 3);
  for (size_t i = 0; i < noise.pixels.size(); ++i) noise.pixels[i] = (uint8_t)((i * 7) ^ (i >> 5));
  const Path file = tmp_file("_test.PNG");
  for (const RgbImage* img : {&red, &noise})
    for (int level : {0, 1}) {
      save_png(img->view(), file, level, 2);
      const RgbImage back = open_png(file);
      CHECK(back.width == img->width && back.height == img->height && back.pixels == img->pixels);
    }
  const std::string junk = "this is not an image";
  {
    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    f << junk;
  }
  bool threw = false;
  try {
    open_png(file);
  } catch (const Error& e) {
    threw = e.code() == MG_ERR_ARG;
  }
  CHECK(threw);
  std::filesystem::remove(file);
  threw = false;
  try {
    open_png(tmp_file("_nonexistent.png"));
  } catch (const Error&) {
    threw = true;
  }
  CHECK(threw);
}

// A w x h grey JPEG written by hand (T.81 baseline): one component, quantiser
// 1, a DC code and an AC code of one symbol each ("0": category 0, "0": EOB),
// so every block holds DC 0 alone and decodes to level 128 everywhere.
static std::vector<uint8_t> grey_jpeg(int w = 16, int h = 8) {
  std::vector<uint8_t> j = {0xFF, 0xD8, 0xFF, 0xDB, 0x00, 0x43, 0x00};
  j.insert(j.end(), 64, 1);
  const uint8_t sof[] = {0xFF, 0xC0, 0x00, 0x0B, 8, (uint8_t)(h >> 8), (uint8_t)h, (uint8_t)(w >> 8), (uint8_t)w,
                         1, 1, 0x11, 0};
  j.insert(j.end(), sof, sof + sizeof(sof));
  const uint8_t dht_head[] = {0xFF, 0xC4, 0x00, 0x26};
  j.insert(j.end(), dht_head, dht_head + 4);
  for (uint8_t cls : {0x00, 0x10}) {
    j.push_back(cls);
    j.push_back(1);  // one code of length 1
    j.insert(j.end(), 15, 0);
    j.push_back(0);  // its symbol
  }
  const uint8_t sos[] = {0xFF, 0xDA, 0x00, 0x08, 1, 1, 0x00, 0, 63, 0};
  j.insert(j.end(), sos, sos + sizeof(sos));
  const int bits = 2 * ((w + 7) / 8) * ((h + 7) / 8);  // "00" per block, then 1-bits to the byte's end
  j.insert(j.end(), (size_t)(bits + 7) / 8, 0);
  if (bits % 8) j.back() = (uint8_t)((1u << (8 - bits % 8)) - 1u);
  j.push_back(0xFF);
  j.push_back(0xD9);
  return j;
}

static void write_bytes(const Path& p, const std::vector<uint8_t>& d) {
  std::ofstream f(p, std::ios::binary | std::ios::trunc);
  f.write(reinterpret_cast<const char*>(d.data()), (std::streamsize)d.size());
}

static RgbImage solid_image(int w, int h, uint8_t r, uint8_t g, uint8_t b) {
  RgbImage img;
  img.width = w;
  img.height = h;
  img.pixels.resize((size_t)w * h * 3);
  for (size_t i = 0; i < img.pixels.size(); i += 3) {
    img.pixels[i] = r;
    img.pixels[i + 1] = g;
    img.pixels[i + 2] = b;
  }
  return img;
}

// main.rs:672 DynamicImage::save: the format from the extension.
static void save_image_tests() {
  const Path dir = tmp_file("_save");
  std::filesystem::remove_all(dir);
  std::filesystem::create_directories(dir);
  RgbImage img = solid_image(37, 21, 0, 0, 0);
  for (int y = 0; y < 21; ++y)
    for (int x = 0; x < 37; ++x) {
      const uint8_t g = (uint8_t)(60 + 3 * x + 2 * y);
      uint8_t* p = img.pixels.data() + 3 * (y * 37 + x);
      p[0] = p[1] = p[2] = g;
    }
  save_image(img.view(), dir / "a.png");
  save_image(img.view(), dir / "b.jpeg");
  save_image(img.view(), dir / "c.JpG");
  CHECK(open_png(dir / "a.png").pixels == img.pixels);
  for (const char* n : {"b.jpeg", "c.JpG"}) {
    const RgbImage back = open_image(dir / n);
    int worst = 0;
    for (size_t i = 0; i < img.pixels.size(); ++i) worst = std::max(worst, std::abs((int)back.pixels[i] - img.pixels[i]));
    CHECK(back.width == 37 && back.height == 21 && worst <= 8);  // grey ramp at quality 75
  }
  CHECK(detail::read_file(dir / "b.jpeg") == encode_jpeg(img.view(), 75));
  bool threw = false;
  try {
    save_image(img.view(), dir / "d.bmp");
  } catch (const Error& e) {
    threw = e.code() == MG_ERR_ARG;
  }
  CHECK(threw && !std::filesystem::exists(dir / "d.bmp"));
  std::filesystem::remove_all(dir);
}

static void material_file_tests() {  // main.rs:166-206 load_tiles' files (extensions, skipped files)
  const Path dir = tmp_file("_materials");
  std::filesystem::remove_all(dir);
  std::filesystem::create_directories(dir / "sub.png");  // a folder with an image extension: not a file
  const RgbImage red = solid_image(4, 3, 255, 0, 0), blue = solid_image(5, 2, 0, 0, 255);
  save_png(red.view(), dir / "a.png", 1, 1);
  save_png(blue.view(), dir / "B.PNG", 0, 1);
  write_bytes(dir / "c.JPG", grey_jpeg());
  write_bytes(dir / "d.webp", {'R', 'I', 'F', 'F', 0, 0, 0, 0, 'W', 'E', 'B', 'P'});
  write_bytes(dir / "e.txt", {'x'});
  const MaterialFiles m = read_material_files(dir, 2);
  CHECK(m.paths.size() == 3 && m.images.size() == 3);
  if (m.paths.size() == 3) {
    CHECK(m.paths[0].filename() == "B.PNG" && m.paths[1].filename() == "a.png" && m.paths[2].filename() == "c.JPG");
    CHECK(m.images[0].pixels == blue.pixels && m.images[1].pixels == red.pixels);
    const RgbImage& g = m.images[2];
    CHECK(g.width == 16 && g.height == 8);
    CHECK(std::all_of(g.pixels.begin(), g.pixels.end(), [](uint8_t v) { return v == 128; }));
  }
  CHECK(m.errors.size() == 1 && m.errors[0].first.filename() == "d.webp");
  const RgbImage j = open_image(dir / "c.JPG");
  CHECK(j.width == 16 && j.height == 8 && j.pixels[0] == 128);
  for (int h : {1, 7, 12, 17}) {  // block counts of every parity: the entropy data ends mid-byte or on a byte
    const std::vector<uint8_t> d = grey_jpeg(24, h);
    const RgbImage g = decode_image(d.data(), d.size());
    CHECK(g.width == 24 && g.height == h);
    CHECK(std::all_of(g.pixels.begin(), g.pixels.end(), [](uint8_t v) { return v == 128; }));
  }
  bool threw = false;
  try {
    open_png(dir / "c.JPG");  // a JPEG is not a PNG
  } catch (const Error& e) {
    threw = e.code() == MG_ERR_ARG;
  }
  CHECK(threw);
  threw = false;
  try {
    read_material_files(dir / "missing");
  } catch (const Error& e) {
    threw = e.code() == MG_ERR_ARG;
  }
  CHECK(threw);
  std::filesystem::remove_all(dir);
}

static void generate_files_tests() {  // main.rs:105-164 + 477-685 from files
  const Path dir = tmp_file("_gen_files");
  std::filesystem::remove_all(dir);
  std::filesystem::create_directories(dir / "materials");
  uint32_t s = 21;
  RgbImage target = solid_image(96, 72, 0, 0, 0);
  for (size_t i = 0; i < target.pixels.size(); ++i) target.pixels[i] = (uint8_t)(lcg(s) >> 24);
  save_png(target.view(), dir / "target.png", 1, 1);
  for (int i = 0; i < 24; ++i) {
    const RgbImage m = solid_image(16, 12, (uint8_t)(lcg(s) >> 24), (uint8_t)(lcg(s) >> 24), (uint8_t)(lcg(s) >> 24));
    save_png(m.view(), dir / "materials" / ("m" + std::to_string(100 + i) + ".png"), 1, 1);
  }
  write_bytes(dir / "materials" / "grey.jpeg", grey_jpeg(16, 12));  // 4:3, as the target: passes the aspect filter
  write_bytes(dir / "materials" / "broken.jpg", {0xFF, 0xD8, 0xFF});
  MosaicOptions o;
  o.grid_w = 12;
  o.grid_h = 9;
  o.max_usage_per_image = 6;
  o.optimization_iterations = 300;
  o.seed = 5;
  std::vector<std::pair<Path, std::string>> skipped;
  const Path out_path = dir / "out" / "deeper" / "mosaic.png";
  const MosaicOutput a = generate_mosaic_files(dir / "target.png", dir / "materials", out_path, o, 2, &skipped);
  CHECK(skipped.size() == 1 && skipped[0].first.filename() == "broken.jpg");
  const MaterialFiles m = read_material_files(dir / "materials");
  const RgbImage t = open_image(dir / "target.png");
  const MosaicOutput b = generate_mosaic(t.view(), m.views(), m.paths, o);
  CHECK(a.palette_size == 25);  // 24 PNGs and the JPEG; the broken file skipped
  CHECK(a.grid == b.grid);
  CHECK(a.image.pixels == b.image.pixels);
  const RgbImage saved = open_png(out_path);
  CHECK(saved.width == 96 && saved.height == 72 && saved.pixels == a.image.pixels);
  // main.rs:672 picks the format by extension: a .jpg path is a JPEG file
  const MosaicOutput j = generate_mosaic_files(dir / "target.png", dir / "materials", dir / "mosaic.JPG", o);
  CHECK(j.image.pixels == a.image.pixels);
  const std::vector<uint8_t> jf = detail::read_file(dir / "mosaic.JPG");
  CHECK(jf.size() > 3 && jf[0] == 0xFF && jf[1] == 0xD8 && jf[2] == 0xFF);
  const RgbImage back = open_image(dir / "mosaic.JPG");
  CHECK(back.width == 96 && back.height == 72);
  bool threw = false;
  try {
    generate_mosaic_files(dir / "target.png", dir / "materials", dir / "mosaic.bmp", o);
  } catch (const Error& e) {
    threw = e.code() == MG_ERR_ARG;
  }
  CHECK(threw);
  std::filesystem::remove_all(dir);
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "--gpu") == 0;
  usage_tracker_tests();
  aspect_tests();
  grid_position_tests();
  lab_distance_tests();
  similarity_host_tests();
  similarity_json_tests();
  color_host_tests();
  result_tests();
  png_tests();
  save_image_tests();
  material_file_tests();
  if (gpu) {
    average_lab_tests();
    similarity_device_tests();
    adjacency_device_tests();
    optimizer_device_tests();
    color_device_tests();
    generate_tests();
    generate_files_tests();
  } else {
    // without a GPU the mirror reports the failure as mosaic::Error
    bool threw = false;
    try {
      Context ctx(0);
    } catch (const Error& e) {
      threw = e.code() != MG_OK;
    }
    CHECK(threw);
  }
  std::printf("%s: %d checks, %d failed\n", gpu ? "gpu" : "cpu", g_checked, g_failed);
  return g_failed == 0 ? 0 : 1;
}

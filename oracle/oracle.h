/*
 * oracle.h -- CPU restatement of mosaic-art-rust's tile matching-and-placement
 * path.  TEST INFRASTRUCTURE ONLY: the test suite, the smoke check and the
 * benchmark's CPU-baseline leg call these functions as the checker.  Nothing in
 * the shipped library links or calls them.
 *
 * Parity status.  The reference is a Rust crate and cannot be built where this
 * oracle is developed (no cargo/rustc), so the oracle is pinned against the
 * reference's own known-answer unit tests (Lab of red and grey, UsageTracker,
 * calculate_average_rgb, similarity symmetry, colour-adjustment clamps and
 * directions, improvement_percentage).  Where the reference's arithmetic lives
 * in third-party crates that are not in the reference tree (palette 0.7.6 for
 * sRGB->Lab and sRGB<->HSV, kiddo 5.2.2 for the k-nearest query, rand 0.8.5 for
 * the annealing stream) the oracle restates the published algorithms; exact
 * last-bit agreement with those crates is unpinned.
 *
 * Every function cites the reference file:line it follows.  Grid cells hold a
 * palette index, -1 meaning "no tile" (the reference's Option<PathBuf> = None).
 */
#ifndef MOSAIC_ORACLE_H
#define MOSAIC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- colour statistics (lib.rs:94-119, main.rs:687-708) ---------------- */
void  orc_srgb_lut(float out[256]);
void  orc_lab_pixel_f64(int r, int g, int b, double out[3]);
void  orc_lab_mean_f64(const uint8_t* rgb, int w, int h, long stride, double out[3]);
void  orc_lab_mean_reffold(const uint8_t* rgb, int w, int h, long stride, float out[3]);
void  orc_lab_pixel_spec(int r, int g, int b, float out[3]);
void  orc_lab_consts(float lut[256], float ms[9], float k[3]);
void  orc_lab_pixels_q(const uint8_t* rgb, long n, int32_t* q);
void  orc_lab_mean_spec(const uint8_t* rgb, int w, int h, long stride, float out[3]);
void  orc_avg_rgb(const uint8_t* rgb, int w, int h, long stride, uint8_t out[3]);
void  orc_resize_lanczos3(const uint8_t* rgb, int w, int h, long stride, int dw, int dh, uint8_t* out);
int   orc_cells(const uint8_t* img, int w, int h, long stride, int gw, int gh,
                float* lab_out, uint8_t* avg_rgb_out);
int   orc_is_aspect_ratio_match(float img_aspect, float target_aspect, float tol);
int   orc_select_palette(const int* widths, const int* heights, int n,
                         float target_aspect, float tol, int max_materials, int* selected);

/* ---- similarity database (similarity.rs:69-146) ------------------------- */
float orc_lab_distance(const float a[3], const float b[3]);
void  orc_similarity_tri(const float* lab, int p, float* out);
void  orc_similarity_full(const float* lab, int p, float* out);

/* ---- k nearest (kiddo nearest_n, main.rs:348-352) ------------------------ */
void  orc_nearest_n(const float* pal, int p, const float q[3], int k, uint32_t* idx, float* dist);

/* ---- adjacency (adjacency.rs:63-214) and placement (main.rs:309-475) ------ */
float orc_penalty(const float* pal, int p, int cand, int x, int y,
                  const int32_t* grid, int gw, int gh, float weight);
float orc_total_cost(const float* pal, int p, const int32_t* grid, int gw, int gh);
float orc_swap_delta(const float* pal, int p, const int32_t* grid, int gw, int gh,
                     int x1, int y1, int x2, int y2);
int   orc_place_greedy(const float* pal, int p, const float* cell_lab, int gw, int gh,
                       int max_usage, float weight, int32_t* grid, int* n_resets);
/* the GUI generator's scoring (gui/app_full.rs:1396-1470): sqrt distance + penalty */
int   orc_place_greedy_gui(const float* pal, int p, const float* cell_lab, int gw, int gh,
                           int max_usage, float weight, int32_t* grid, int* n_resets);

/* ---- annealing (optimizer.rs:41-129) -------------------------------------- */
void  orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
float orc_exp(float x);
/* res: [initial, final, best]; counts: [accepted, improved, cooled iterations] */
void  orc_anneal(const float* pal, int p, int32_t* grid, int gw, int gh, long iters,
                 float t0, float decay, uint64_t seed, uint32_t stream, uint32_t chain,
                 int greedy_only, float res[3], int64_t counts[3]);

/* ---- colour adjustment (color_adjustment.rs:30-154) ---------------------- */
void  orc_rgb_to_hsv(float r, float g, float b, float out[3]);
void  orc_hsv_to_rgb(float h, float s, float v, float out[3]);
void  orc_adjustment_new(float br, float co, float hue, float sat, float out[4]);
void  orc_optimal_adjustment(const uint8_t tile[3], const uint8_t target[3], float strength,
                             float out[4]);
void  orc_adjust_pixel(const float adj[4], const uint8_t in[3], uint8_t out[3]);
void  orc_adjust_pixels(const float adj[4], const uint8_t* in, long n, uint8_t* out);

/* ---- composite (main.rs:583-592, 627-664) -------------------------------- */
void  orc_anneal_ex(const float* pal, int p, int32_t* grid, int gw, int gh, long iters, float t0, float decay,
                    uint64_t seed, uint32_t stream, uint32_t chain, int greedy_only, int libm_exp, float res[3],
                    int64_t counts[3]);
int   orc_composite(const int32_t* grid, int gw, int gh, const uint8_t* thumbs, int tw, int th,
                    const uint8_t* cell_avg_rgb, const uint8_t* thumb_avg_rgb,
                    float strength, uint8_t* out);

/* ---- whole generate_mosaic job (main.rs:105-164, 477-685) ----------------- */
typedef struct orc_job {
  /* target */
  const uint8_t* target; int tw_img, th_img; long tstride;
  /* materials, concatenated; mat_off[i] = byte offset of material i */
  const uint8_t* mats; const int64_t* mat_off; const int* mat_w; const int* mat_h; int n_mats;
  /* thumbnails: n_mats x (thumb_h x thumb_w x 3), indexed by ORIGINAL material index */
  const uint8_t* thumbs; int thumb_w, thumb_h;
  int gw, gh;
  int max_materials; float aspect_tol;
  int max_usage; float weight; float color_strength;
  int enable_opt; long iters; float t0, decay; int chains; uint64_t seed; uint32_t stream;
  int threads;
  int gui_scoring;  /* 1: the GUI generator's scoring (orc_place_greedy_gui) */
  int ref_arith;    /* 1: Lab by the reference's FP32 fold (orc_lab_mean_reffold) and
                       annealing acceptance by libm expf, instead of the defined arithmetic */
} orc_job;

typedef struct orc_out {
  int32_t* grid;          /* N, ORIGINAL material index or -1 */
  uint8_t* image;         /* (gw*thumb_w) x (gh*thumb_h) x 3 */
  float* pal_lab;         /* optional, n_mats*3: palette Lab of the selected materials */
  float* cell_lab;        /* optional, N*3 */
  int32_t* greedy_grid;   /* optional, N, palette index */
  float* chain_res;       /* optional, chains*3 */
  int p;                  /* selected palette size */
  int n_resets;
  int best_chain;
  float initial_cost, final_cost, best_cost;
} orc_out;

int orc_generate(const orc_job* job, orc_out* out);

#ifdef __cplusplus
}
#endif
#endif

/*
 * CPU oracle for the CT reconstruction hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference library's CPU implementations
 * (the .cc files under CT_RECON_EXTENSIONS src/).  It is the checker that the CUDA kernels of
 * ct_recon_extensions_gb300 are compared against, and the CPU baseline that
 * bench.py times.  Nothing in the product path links or calls it: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm.
 *
 * Every function follows the reference's arithmetic in the same order
 * (double geometry, double accumulation where the reference accumulates in
 * double, T accumulation where it accumulates in T), so that compiled with
 * -ffp-contract=off it reproduces the reference's results bit for bit.  The
 * pin is tests/test_oracle_golden.py: fixtures in tests/golden/ were produced
 * by the reference's own src/ sources compiled as they are (oracle/Makefile, target
 * "ref"), and the restatement must match them exactly.
 *
 * Two functions are restatements of the MATH of a reference function rather
 * than of its code, because the reference code is broken there:
 *   - orc_bp_par_2d_grad_*: the reference ParallelBackprojection2DPixDrivenGrad
 *     (src/bp_par_2d.cc:145-199) reads uninitialised pointers.  The oracle is
 *     the exact transpose of the forward bp_par_2d (src/bp_par_2d.cc:51-90).
 *   - orc_bp_fan_2d_angle_grad_*: the reference grad (src/bp_fan_2d_angle.cc:
 *     124-169) divides by the weights and leaves ypos uninitialised.  The
 *     oracle is the exact transpose of the angle BP, built on the scatter of
 *     src/bp_fan_2d.cc:124-173 with no orbit scale.
 *
 * Row-range variants (_rows) compute output rows [r0, r1) only; they let a
 * caller run disjoint row ranges on several host threads with results
 * identical to the single-threaded call.
 */
#ifndef CTR_ORACLE_H
#define CTR_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Geometry shared by the fan and parallel operators (superset of the
 * reference Param structs; each function reads the fields it needs). */
typedef struct orc_geom {
    unsigned int ns, na;
    double ds, orbit, offset_s, orbit_start;
    unsigned int nx, ny;
    double dx, dy, offset_x, offset_y;
    double dso, dsd, fov;
} orc_geom;

/* ---- fan weighting: src/fan_weighting.cc:19-59 ---- */
int orc_fan_weighting_f32(unsigned ns, unsigned nrow, double ds, double offset,
                          double dso, double dsd, int type, const float* in, float* out);
int orc_fan_weighting_f64(unsigned ns, unsigned nrow, double ds, double offset,
                          double dso, double dsd, int type, const double* in, double* out);
/* the reference grad applies the same diagonal weight (src/fan_weighting.cc:40-59) */
int orc_fan_weighting_grad_f32(unsigned ns, unsigned nrow, double ds, double offset,
                               double dso, double dsd, int type, const float* in, float* out);
int orc_fan_weighting_grad_f64(unsigned ns, unsigned nrow, double ds, double offset,
                               double dso, double dsd, int type, const double* in, double* out);

/* ---- ramp filter: src/filter.cc:18-124 ---- */
/* filter has 2*ns+1 taps, tap n at filter[n+ns] */
int orc_ramp_filter_prep(unsigned ns, double ds, double dsd, int type, double* filter);
int orc_ramp_filter_rows_f32(unsigned ns, unsigned r0, unsigned r1, double ds,
                             const float* in, const double* filter, float* out);
int orc_ramp_filter_rows_f64(unsigned ns, unsigned r0, unsigned r1, double ds,
                             const double* in, const double* filter, double* out);
int orc_ramp_filter_grad_rows_f32(unsigned ns, unsigned r0, unsigned r1, double ds,
                                  const float* in, const double* filter, float* out);
int orc_ramp_filter_grad_rows_f64(unsigned ns, unsigned r0, unsigned r1, double ds,
                                  const double* in, const double* filter, double* out);

/* ---- fan backprojection, uniform orbit: src/bp_fan_2d.cc:18-173 ---- */
int orc_bp_fan_2d_prep(const orc_geom* g, double* xpos, double* ypos, double* sincostbl);
int orc_bp_fan_2d_rows_f32(const orc_geom* g, unsigned y0, unsigned y1, const float* proj,
                           float* img, const double* xpos, const double* ypos,
                           const double* sincostbl);
int orc_bp_fan_2d_rows_f64(const orc_geom* g, unsigned y0, unsigned y1, const double* proj,
                           double* img, const double* xpos, const double* ypos,
                           const double* sincostbl);
/* scatter adjoint, accumulates in T exactly as the reference does */
int orc_bp_fan_2d_grad_f32(const orc_geom* g, const float* img, float* grad,
                           const double* xpos, const double* ypos, const double* sincostbl);
int orc_bp_fan_2d_grad_f64(const orc_geom* g, const double* img, double* grad,
                           const double* xpos, const double* ypos, const double* sincostbl);

/* ---- fan backprojection, explicit angles: src/bp_fan_2d_angle.cc:18-91 ---- */
int orc_bp_fan_2d_angle_prep(const orc_geom* g, const double* angles, double* xpos,
                             double* ypos, double* sincostbl);
int orc_bp_fan_2d_angle_rows_f32(const orc_geom* g, unsigned y0, unsigned y1,
                                 const float* proj, float* img, const double* xpos,
                                 const double* ypos, const double* sincostbl);
int orc_bp_fan_2d_angle_rows_f64(const orc_geom* g, unsigned y0, unsigned y1,
                                 const double* proj, double* img, const double* xpos,
                                 const double* ypos, const double* sincostbl);
int orc_bp_fan_2d_angle_grad_f32(const orc_geom* g, const float* img, float* grad,
                                 const double* xpos, const double* ypos,
                                 const double* sincostbl);
int orc_bp_fan_2d_angle_grad_f64(const orc_geom* g, const double* img, double* grad,
                                 const double* xpos, const double* ypos,
                                 const double* sincostbl);

/* ---- parallel backprojection: src/bp_par_2d.cc:18-90 ---- */
/* xcos is [nx][na], ysin is [ny][na] */
int orc_bp_par_2d_prep(const orc_geom* g, double* xcos, double* ysin);
int orc_bp_par_2d_rows_f32(const orc_geom* g, unsigned y0, unsigned y1, const float* proj,
                           float* img, const double* xcos, const double* ysin);
int orc_bp_par_2d_rows_f64(const orc_geom* g, unsigned y0, unsigned y1, const double* proj,
                           double* img, const double* xcos, const double* ysin);
/* exact transpose of bp_par_2d (double accumulation, cast at the end) */
int orc_bp_par_2d_grad_f32(const orc_geom* g, const float* img, float* grad,
                           const double* xcos, const double* ysin);
int orc_bp_par_2d_grad_f64(const orc_geom* g, const double* img, double* grad,
                           const double* xcos, const double* ysin);

/* ---- parallel single-view backprojection: src/bp_par_2d_sv.cc:18-92 ---- */
/* img is [ny][nx][na] */
int orc_bp_par_2d_sv_rows_f32(const orc_geom* g, unsigned y0, unsigned y1, const float* proj,
                              float* img, const double* xcos, const double* ysin);
int orc_bp_par_2d_sv_rows_f64(const orc_geom* g, unsigned y0, unsigned y1, const double* proj,
                              double* img, const double* xcos, const double* ysin);

/* ---- parallel ray-driven forward projection: src/fp_par_2d.cc:149-391 ---- */
/* sincostbl [na][2], beginoffset [na][ns][2], usex [na] */
int orc_fp_par_2d_prep(const orc_geom* g, double* sincostbl, double* beginoffset, int* usex);
int orc_fp_par_2d_views_f32(const orc_geom* g, unsigned a0, unsigned a1, const float* img,
                            float* proj, const double* sincostbl, const double* beginoffset,
                            const int* usex);
int orc_fp_par_2d_views_f64(const orc_geom* g, unsigned a0, unsigned a1, const double* img,
                            double* proj, const double* sincostbl, const double* beginoffset,
                            const int* usex);
/* weights [na], pos [na][max(nx,ny)][2], usex [na] */
int orc_fp_par_2d_grad_prep(const orc_geom* g, double* weights, double* pos, int* usex);
int orc_fp_par_2d_grad_rows_f32(const orc_geom* g, unsigned y0, unsigned y1, const float* proj,
                                float* img, const double* weights, const double* pos,
                                const int* usex);
int orc_fp_par_2d_grad_rows_f64(const orc_geom* g, unsigned y0, unsigned y1,
                                const double* proj, double* img, const double* weights,
                                const double* pos, const int* usex);

/* ---- parallel ray-casting FP: src/fp_par_2d.cc:18-145 ---- */
int orc_fp_par_2d_cast_prep(const orc_geom* g, double step_size, double* sincostbl, double* begins,
                            int* nsteps);
int orc_fp_par_2d_cast_views_f32(const orc_geom* g, unsigned a0, unsigned a1, double step_size,
                                 const float* img, float* proj, const double* sincostbl,
                                 const double* begins, const int* nsteps);
int orc_fp_par_2d_cast_views_f64(const orc_geom* g, unsigned a0, unsigned a1, double step_size,
                                 const double* img, double* proj, const double* sincostbl,
                                 const double* begins, const int* nsteps);

/* ---- parallel distance-driven FP and its reference grad: src/fp_par_2d.cc:396-653 ---- */
int orc_fp_par_2d_dd_prep(const orc_geom* g, double* sincostbl, double* beginoffset, int* usex);
int orc_fp_par_2d_dd_grad_prep(const orc_geom* g, double* weights, double* pos, int* usex);
int orc_fp_par_2d_dd_views_f32(const orc_geom* g, unsigned a0, unsigned a1, const float* img,
                               float* proj, const double* sincostbl, const double* beginoffset,
                               const int* usex);
int orc_fp_par_2d_dd_views_f64(const orc_geom* g, unsigned a0, unsigned a1, const double* img,
                               double* proj, const double* sincostbl, const double* beginoffset,
                               const int* usex);
int orc_fp_par_2d_dd_grad_rows_f32(const orc_geom* g, unsigned y0, unsigned y1, const float* proj,
                                   float* img, const double* weights, const double* pos,
                                   const int* usex);
int orc_fp_par_2d_dd_grad_rows_f64(const orc_geom* g, unsigned y0, unsigned y1, const double* proj,
                                   double* img, const double* weights, const double* pos,
                                   const int* usex);

/* ---- helical rebinning: src/helical_interpolation.cc:80-370 ----
 * Field order of HelicalInterpolationParam (include/helical_interpolation.h:17-64).
 * Input [na][nt][ns] (view, detector row, channel), output [nz][view_per_rot][ns].
 * Slices [z0, z1) of the reference's calculate_on_cpu loop (slice iz sits at
 * z0 + dz added iz times).  Returns 1, or 3 when a 180LI corresponding-view
 * sample fell outside the scan's views and read as 0 (the reference reads out
 * of bounds there); ORC_HELI_ERR_VIEWS / ORC_HELI_ERR_ROWS where the
 * reference throws "View not enough for this slice!" / "No row data
 * available!" (the output rows before that point are written, as in the
 * reference). */
typedef struct orc_heli {
    unsigned int ns, nt, na;
    double ds, dt, offset_s, offset_t, orbit_start, orbit, couch_begin, couch_mov;
    unsigned int view_per_rot, nz;
    double dz, z0, thickness, dso, dsd;
} orc_heli;
#define ORC_HELI_ERR_VIEWS (-1)
#define ORC_HELI_ERR_ROWS (-2)
int orc_helical_360_slices_f32(const orc_heli* h, unsigned z0, unsigned z1, const float* in, float* out);
int orc_helical_360_slices_f64(const orc_heli* h, unsigned z0, unsigned z1, const double* in, double* out);
int orc_helical_180_slices_f32(const orc_heli* h, unsigned z0, unsigned z1, const float* in, float* out);
int orc_helical_180_slices_f64(const orc_heli* h, unsigned z0, unsigned z1, const double* in, double* out);

#ifdef __cplusplus
}
#endif
#endif

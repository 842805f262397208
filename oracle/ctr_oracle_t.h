/*
 * T-generic body of the CPU oracle (test infrastructure only).  Included by
 * ctr_oracle.c twice, with T = float / SFX = f32 and T = double / SFX = f64,
 * which stands in for the reference's explicit template instantiations
 * (e.g. src/bp_fan_2d.cc:93-94).
 */
#define ORC_CAT2(a, b) a##_##b
#define ORC_CAT(a, b) ORC_CAT2(a, b)
#define ORC_FN(name) ORC_CAT(name, SFX)

/* src/fan_weighting.cc:19-38 */
static int ORC_FN(fan_weight_apply)(unsigned ns, unsigned nrow, double ds, double offset,
                                    double dso, double dsd, int type, const T* in, T* out,
                                    int weight_first)
{
    const double cents = (double)(ns - 1) / 2 + offset;
    for (unsigned is = 0; is < ns; ++is) {
        const double s = ds * ((double)is - cents);
        double w;
        if (type == 2)
            w = dso * fabs(cos(atan2(s, dsd))) / dsd;
        else if (type == 1)
            w = dso * fabs(cos(s / dsd)) / dsd;
        else
            return 0;
        for (unsigned ia = 0; ia < nrow; ++ia) {
            const size_t k = (size_t)is + (size_t)ia * ns;
            out[k] = weight_first ? (T)(w * in[k]) : (T)(in[k] * w);
        }
    }
    return 1;
}

int ORC_FN(orc_fan_weighting)(unsigned ns, unsigned nrow, double ds, double offset,
                              double dso, double dsd, int type, const T* in, T* out)
{
    return ORC_FN(fan_weight_apply)(ns, nrow, ds, offset, dso, dsd, type, in, out, 1);
}

/* src/fan_weighting.cc:40-59 */
int ORC_FN(orc_fan_weighting_grad)(unsigned ns, unsigned nrow, double ds, double offset,
                                   double dso, double dsd, int type, const T* in, T* out)
{
    return ORC_FN(fan_weight_apply)(ns, nrow, ds, offset, dso, dsd, type, in, out, 0);
}

/* src/filter.cc:67-91: linear (zero-padded) convolution with the 2ns+1 taps */
int ORC_FN(orc_ramp_filter_rows)(unsigned ns, unsigned r0, unsigned r1, double ds,
                                 const T* in, const double* filter, T* out)
{
    const double* h = filter + ns;
    const int n = (int)ns;
    for (unsigned r = r0; r < r1; ++r) {
        const T* row = in + (size_t)r * ns;
        T* orow = out + (size_t)r * ns;
        for (int i = 0; i < n; ++i) {
            double acc = 0;
            for (int k = -n; k <= n; ++k) {
                const int j = i - k;
                if (j >= 0 && j < n) acc += row[j] * h[k];
            }
            orow[i] = (T)(acc * ds);
        }
    }
    return 1;
}

/* src/filter.cc:96-124: correlation, zero taps skipped as in the reference */
int ORC_FN(orc_ramp_filter_grad_rows)(unsigned ns, unsigned r0, unsigned r1, double ds,
                                      const T* in, const double* filter, T* out)
{
    const double* h = filter + ns;
    const int n = (int)ns;
    for (unsigned r = r0; r < r1; ++r) {
        const T* row = in + (size_t)r * ns;
        T* orow = out + (size_t)r * ns;
        for (int i = 0; i < n; ++i) {
            double acc = 0;
            for (int k = -n; k <= n; ++k) {
                const int j = i + k;
                if (j >= 0 && j < n && (h[k] > 0 || h[k] < 0)) acc += row[j] * h[k];
            }
            orow[i] = (T)(acc * ds);
        }
    }
    return 1;
}

/* One fan-beam pixel-view term of src/bp_fan_2d.cc:66-82.  Returns 1 when the
 * projected channel lies on the detector, with the interpolation taps and
 * the distance weight. */
static int ORC_FN(fan_tap)(const orc_geom* g, double x, double y, double sb, double cb,
                           double cents, unsigned* is1, unsigned* is2, double* u,
                           double* w)
{
    const double d = g->dso + x * sb - y * cb;
    const double r = x * cb + y * sb;
    const double gamma = atan2(r, d);
    const double s = gamma * g->dsd / g->ds + cents;
    *w = g->dsd * g->dsd / (d * d + r * r);
    if (s >= 0 && s <= g->ns - 1) {
        *is1 = (unsigned)floor(s);
        *is2 = (unsigned)ceil(s);
        *u = s - *is1;
        return 1;
    }
    return 0;
}

/* Gather over views for output rows [y0, y1) (src/bp_fan_2d.cc:46-91 with
 * scale = |orbit|/F, and src/bp_fan_2d_angle.cc:47-91 with no scale). */
static void ORC_FN(fan_bp_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                                T* img, const double* xpos, const double* ypos,
                                const double* sc, int scaled)
{
    const double cents = (double)(g->ns - 1) / 2 + g->offset_s;
    const double factor = round(fabs(g->na * g->orbit) / M_PI);
    for (unsigned iy = y0; iy < y1; ++iy) {
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            double sum = 0.0;
            for (unsigned ia = 0; ia < g->na; ++ia) {
                unsigned is1, is2;
                double u, w;
                if (ORC_FN(fan_tap)(g, xpos[ix], ypos[iy], sc[2 * ia], sc[2 * ia + 1], cents,
                                    &is1, &is2, &u, &w)) {
                    const T* p = proj + (size_t)ia * g->ns;
                    sum += ((1 - u) * p[is1] + u * p[is2]) * w;
                }
            }
            img[(size_t)iy * g->nx + ix] =
                scaled ? (T)(sum * fabs(g->orbit) / factor) : (T)sum;
        }
    }
}

int ORC_FN(orc_bp_fan_2d_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                               T* img, const double* xpos, const double* ypos,
                               const double* sincostbl)
{
    ORC_FN(fan_bp_rows)(g, y0, y1, proj, img, xpos, ypos, sincostbl, 1);
    return 1;
}

int ORC_FN(orc_bp_fan_2d_angle_rows)(const orc_geom* g, unsigned y0, unsigned y1,
                                     const T* proj, T* img, const double* xpos,
                                     const double* ypos, const double* sincostbl)
{
    ORC_FN(fan_bp_rows)(g, y0, y1, proj, img, xpos, ypos, sincostbl, 0);
    return 1;
}

/* Scatter adjoint of the fan BP (src/bp_fan_2d.cc:124-173): taps are cast to T
 * and accumulated into the T output, then scaled by |orbit|/F when scaled. */
static void ORC_FN(fan_bp_grad)(const orc_geom* g, const T* img, T* grad, const double* xpos,
                                const double* ypos, const double* sc, int scaled)
{
    const double cents = (double)(g->ns - 1) / 2 + g->offset_s;
    const double factor = round(fabs(g->na * g->orbit) / M_PI);
    const size_t n = (size_t)g->ns * g->na;
    for (size_t i = 0; i < n; ++i) grad[i] = 0;
    for (unsigned iy = 0; iy < g->ny; ++iy) {
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            const T v = img[(size_t)iy * g->nx + ix];
            for (unsigned ia = 0; ia < g->na; ++ia) {
                unsigned is1, is2;
                double u, w;
                if (ORC_FN(fan_tap)(g, xpos[ix], ypos[iy], sc[2 * ia], sc[2 * ia + 1], cents,
                                    &is1, &is2, &u, &w)) {
                    T* gr = grad + (size_t)ia * g->ns;
                    gr[is1] += v * (T)(w * (1 - u));
                    gr[is2] += v * (T)(w * u);
                }
            }
        }
    }
    if (scaled) {
        const T weight = (T)(fabs(g->orbit) / factor);
        for (size_t i = 0; i < n; ++i) grad[i] *= weight;
    }
}

int ORC_FN(orc_bp_fan_2d_grad)(const orc_geom* g, const T* img, T* grad, const double* xpos,
                               const double* ypos, const double* sincostbl)
{
    ORC_FN(fan_bp_grad)(g, img, grad, xpos, ypos, sincostbl, 1);
    return 1;
}

int ORC_FN(orc_bp_fan_2d_angle_grad)(const orc_geom* g, const T* img, T* grad,
                                     const double* xpos, const double* ypos,
                                     const double* sincostbl)
{
    ORC_FN(fan_bp_grad)(g, img, grad, xpos, ypos, sincostbl, 0);
    return 1;
}

/* One parallel-beam pixel-view term of src/bp_par_2d.cc:70-76. */
static int ORC_FN(par_tap)(const orc_geom* g, double xc, double ys, double cents,
                           unsigned* is1, unsigned* is2, double* u)
{
    const double s = (xc + ys) / g->ds + cents;
    if (s >= 0 && s <= g->ns - 1) {
        *is1 = (unsigned)floor(s);
        *is2 = (unsigned)ceil(s);
        *u = s - *is1;
        return 1;
    }
    return 0;
}

/* src/bp_par_2d.cc:51-90: signed orbit scale */
int ORC_FN(orc_bp_par_2d_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                               T* img, const double* xcos, const double* ysin)
{
    const double cents = (double)(g->ns - 1) / 2 + g->offset_s;
    for (unsigned iy = y0; iy < y1; ++iy) {
        const double* ys = ysin + (size_t)iy * g->na;
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            const double* xc = xcos + (size_t)ix * g->na;
            double sum = 0.0;
            for (unsigned ia = 0; ia < g->na; ++ia) {
                unsigned is1, is2;
                double u;
                if (ORC_FN(par_tap)(g, xc[ia], ys[ia], cents, &is1, &is2, &u)) {
                    const T* p = proj + (size_t)ia * g->ns;
                    sum += (1 - u) * p[is1] + u * p[is2];
                }
            }
            img[(size_t)iy * g->nx + ix] = (T)(sum * g->orbit);
        }
    }
    return 1;
}

/* Exact transpose of orc_bp_par_2d_rows: every tap of the forward gather is
 * scattered back with the same weight; double accumulation, orbit applied
 * once at the end. */
int ORC_FN(orc_bp_par_2d_grad)(const orc_geom* g, const T* img, T* grad, const double* xcos,
                               const double* ysin)
{
    const double cents = (double)(g->ns - 1) / 2 + g->offset_s;
    const size_t n = (size_t)g->ns * g->na;
    double* acc = (double*)calloc(n, sizeof(double));
    if (!acc) return 0;
    for (unsigned iy = 0; iy < g->ny; ++iy) {
        const double* ys = ysin + (size_t)iy * g->na;
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            const double* xc = xcos + (size_t)ix * g->na;
            const double v = img[(size_t)iy * g->nx + ix];
            for (unsigned ia = 0; ia < g->na; ++ia) {
                unsigned is1, is2;
                double u;
                if (ORC_FN(par_tap)(g, xc[ia], ys[ia], cents, &is1, &is2, &u)) {
                    double* a = acc + (size_t)ia * g->ns;
                    a[is1] += (1 - u) * v;
                    a[is2] += u * v;
                }
            }
        }
    }
    for (size_t i = 0; i < n; ++i) grad[i] = (T)(acc[i] * g->orbit);
    free(acc);
    return 1;
}

/* src/bp_par_2d_sv.cc:55-92: one lerp value per view, 0 off the detector */
int ORC_FN(orc_bp_par_2d_sv_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                                  T* img, const double* xcos, const double* ysin)
{
    const double cents = (double)(g->ns - 1) / 2 + g->offset_s;
    for (unsigned iy = y0; iy < y1; ++iy) {
        const double* ys = ysin + (size_t)iy * g->na;
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            const double* xc = xcos + (size_t)ix * g->na;
            T* o = img + ((size_t)iy * g->nx + ix) * g->na;
            for (unsigned ia = 0; ia < g->na; ++ia) {
                unsigned is1, is2;
                double u;
                if (ORC_FN(par_tap)(g, xc[ia], ys[ia], cents, &is1, &is2, &u)) {
                    const T* p = proj + (size_t)ia * g->ns;
                    o[ia] = (T)((1 - u) * p[is1] + u * p[is2]);
                } else {
                    o[ia] = 0;
                }
            }
        }
    }
    return 1;
}

/* src/fp_par_2d.cc:210-280: ray-driven projection of views [a0, a1); the ray
 * sum accumulates in T exactly as the reference does (T sum). */
int ORC_FN(orc_fp_par_2d_views)(const orc_geom* g, unsigned a0, unsigned a1, const T* img,
                                T* proj, const double* sincostbl, const double* beginoffset,
                                const int* usex)
{
    for (unsigned ia = a0; ia < a1; ++ia) {
        const double* bo = beginoffset + (size_t)ia * g->ns * 2;
        T* out = proj + (size_t)ia * g->ns;
        if (usex[ia]) {
            const double dist_weight = fabs(g->dy / sincostbl[2 * ia + 1]);
            for (unsigned is = 0; is < g->ns; ++is) {
                double x = bo[2 * is];
                const double step = bo[2 * is + 1];
                T sum = 0;
                for (unsigned iy = 0; iy < g->ny; ++iy) {
                    if (x >= 0 && x <= g->nx - 1) {
                        const unsigned ix1 = (unsigned)floor(x);
                        const unsigned ix2 = (unsigned)ceil(x);
                        const double u = x - ix1;
                        const T* row = img + (size_t)iy * g->nx;
                        sum += (1 - u) * row[ix1] + u * row[ix2];
                    }
                    x += step;
                }
                out[is] = (T)(sum * dist_weight);
            }
        } else {
            const double dist_weight = fabs(g->dx / sincostbl[2 * ia]);
            for (unsigned is = 0; is < g->ns; ++is) {
                double y = bo[2 * is];
                const double step = bo[2 * is + 1];
                T sum = 0;
                for (unsigned ix = 0; ix < g->nx; ++ix) {
                    if (y >= 0 && y <= g->ny - 1) {
                        const unsigned iy1 = (unsigned)floor(y);
                        const unsigned iy2 = (unsigned)ceil(y);
                        const double u = y - iy1;
                        sum += (1 - u) * img[ix + (size_t)iy1 * g->nx] +
                               u * img[ix + (size_t)iy2 * g->nx];
                    }
                    y += step;
                }
                out[is] = (T)(sum * dist_weight);
            }
        }
    }
    return 1;
}

/* src/fp_par_2d.cc:82-145: ray casting of views [a0, a1).  Positions run as
 * FP64 sums from the entry point; a sample inside [0, nx-1] x [0, ny-1] adds
 * the bilinear interpolation (floor / ceil corners) to a double sum, scaled by
 * step_size * dx at the end. */
int ORC_FN(orc_fp_par_2d_cast_views)(const orc_geom* g, unsigned a0, unsigned a1, double step_size,
                                     const T* img, T* proj, const double* sincostbl,
                                     const double* begins, const int* nsteps)
{
    const double xmax = (double)g->nx - 1, ymax = (double)g->ny - 1;
    for (unsigned ia = a0; ia < a1; ++ia) {
        const double sx = step_size * sincostbl[2 * ia], sy = step_size * sincostbl[2 * ia + 1];
        for (unsigned is = 0; is < g->ns; ++is) {
            const size_t r = (size_t)ia * g->ns + is;
            const int nstep = nsteps[r];
            if (nstep <= 0) {
                proj[r] = 0;
                continue;
            }
            double x = begins[2 * r], y = begins[2 * r + 1], sum = 0;
            for (int k = 0; k < nstep; ++k) {
                if (x >= 0 && x <= xmax && y >= 0 && y <= ymax) {
                    const int ix1 = (int)floor(x), ix2 = (int)ceil(x);
                    const int iy1 = (int)floor(y), iy2 = (int)ceil(y);
                    const double u = x - ix1, v = y - iy1;
                    const T* r1 = img + (size_t)iy1 * g->nx;
                    const T* r2 = img + (size_t)iy2 * g->nx;
                    sum += (1 - v) * ((1 - u) * r1[ix1] + u * r1[ix2]) +
                           v * ((1 - u) * r2[ix1] + u * r2[ix2]);
                }
                x += sx;
                y += sy;
            }
            proj[r] = (T)(sum * step_size * g->dx);
        }
    }
    return 1;
}

/* src/fp_par_2d.cc:455-540: distance-driven projection of views [a0, a1).
 * Per line of the marched axis, the footprint [left, right] (running FP64
 * sums) averages the trapezoid of neighbouring pixel pairs over the pixel
 * intervals it covers, in T.  The reference runs the pixel loop with an
 * unsigned index from floor(left); a negative floor converts (undefined in
 * C++) to a huge unsigned on the x86-64 builds the fixtures come from, so such
 * a line contributes nothing: written out here as that rule. */
int ORC_FN(orc_fp_par_2d_dd_views)(const orc_geom* g, unsigned a0, unsigned a1, const T* img,
                                   T* proj, const double* sincostbl, const double* beginoffset,
                                   const int* usex)
{
    for (unsigned ia = a0; ia < a1; ++ia) {
        const double* bo = beginoffset + (size_t)ia * g->ns * 3;
        const int ux = usex[ia];
        const double w = ux ? fabs(g->dy / sincostbl[2 * ia + 1]) : fabs(g->dx / sincostbl[2 * ia]);
        const unsigned nl = ux ? g->ny : g->nx;     /* lines */
        const unsigned na_ = ux ? g->nx : g->ny;    /* pixels along a line */
        for (unsigned is = 0; is < g->ns; ++is) {
            const double c = bo[3 * is], off = bo[3 * is + 1], hw = bo[3 * is + 2];
            double left = c - hw, right = c + hw;
            if (left > right) {
                const double t = left;
                left = right;
                right = t;
            }
            T sum = 0;
            for (unsigned l = 0; l < nl; ++l) {
                T tsum = 0, lsum = 0;
                const double fl = floor(left), cr = ceil(right);
                if (fl >= 0) {
                    for (unsigned i = (unsigned)fl; (double)i < cr; ++i) {
                        if (i >= na_ - 1) continue;
                        const double a = (double)(i + 1) < right ? (double)(i + 1) : right;
                        const double b = (double)i > left ? (double)i : left;
                        const double len = a - b;
                        const T p0 = ux ? img[i + (size_t)l * g->nx] : img[l + (size_t)i * g->nx];
                        const T p1 = ux ? img[i + 1 + (size_t)l * g->nx] : img[l + (size_t)(i + 1) * g->nx];
                        tsum += len * (p0 + p1) / 2;
                        lsum += len;
                    }
                }
                if (lsum > 0) sum += tsum / lsum;
                left += off;
                right += off;
            }
            proj[(size_t)ia * g->ns + is] = (T)(sum * w);
        }
    }
    return 1;
}

/* src/fp_par_2d.cc:598-653: the reference's distance-driven "gradient", rows
 * [y0, y1) of the image (not the adjoint of the forward above: that one
 * normalises by the covered length).  Per pixel and view the channel footprint
 * [left, right] around the pixel's channel; the channel loop's unsigned index
 * from ceil(left - 0.5) skips the view when that is negative (see above), and
 * channels past ns read on into the following view's row, as the reference's
 * unchecked index does (0 past the last view). */
int ORC_FN(orc_fp_par_2d_dd_grad_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                                       T* img, const double* weights, const double* pos,
                                       const int* usex)
{
    const size_t total = (size_t)g->na * g->ns;
    for (unsigned iy = y0; iy < y1; ++iy) {
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            double sum = 0.0;
            for (unsigned ia = 0; ia < g->na; ++ia) {
                const double* pp = pos + (size_t)ia * g->nx * 2;
                double mid, left, right;
                if (usex[ia]) {
                    const double begin = pp[2 * iy], off = pp[2 * iy + 1];
                    mid = begin + off * ix;
                    left = ix == 0 ? mid : mid - off;
                    right = ix == g->nx - 1 ? mid : mid + off;
                } else {
                    const double begin = pp[2 * ix], off = pp[2 * ix + 1];
                    mid = begin + off * iy;
                    left = iy == 0 ? mid : mid - off;
                    right = iy == g->ny - 1 ? mid : mid + off;
                }
                if (left > right) {
                    const double t = left;
                    left = right;
                    right = t;
                }
                double tmp = 0.0;
                const double c0 = ceil(left - 0.5), c1 = floor(right + 0.5);
                if (c0 >= 0) {
                    for (unsigned is = (unsigned)c0; (double)is <= c1; ++is) {
                        const double a = (double)is + 0.5 < right ? (double)is + 0.5 : right;
                        const double b = (double)is - 0.5 > left ? (double)is - 0.5 : left;
                        const size_t k = (size_t)ia * g->ns + is;
                        tmp += (a - b) * (k < total ? proj[k] : 0) / 2;
                    }
                }
                sum += tmp * weights[ia];
            }
            img[(size_t)iy * g->nx + ix] = (T)sum;
        }
    }
    return 1;
}

/* src/fp_par_2d.cc:323-391: per-pixel gather over each view's channel
 * footprint (triangle weights), rows [y0, y1) of the image. */
int ORC_FN(orc_fp_par_2d_grad_rows)(const orc_geom* g, unsigned y0, unsigned y1, const T* proj,
                                    T* img, const double* weights, const double* pos,
                                    const int* usex)
{
    for (unsigned iy = y0; iy < y1; ++iy) {
        for (unsigned ix = 0; ix < g->nx; ++ix) {
            double sum = 0.0;
            for (unsigned ia = 0; ia < g->na; ++ia) {
                const double* pp = pos + (size_t)ia * 2 * g->nx;
                const T* pr = proj + (size_t)ia * g->ns;
                double begin, step, mid, left, right;
                if (usex[ia]) {
                    begin = pp[2 * iy];
                    step = pp[2 * iy + 1];
                    mid = begin + step * ix;
                    left = ix == 0 ? mid : mid - step;
                    right = ix == g->nx - 1 ? mid : mid + step;
                } else {
                    begin = pp[2 * ix];
                    step = pp[2 * ix + 1];
                    mid = begin + step * iy;
                    left = iy == 0 ? mid : mid - step;
                    right = iy == g->ny - 1 ? mid : mid + step;
                }
                if (left > right) {
                    const double t = left;
                    left = right;
                    right = t;
                }
                /* The reference loops is from ceil(left) while is <= right
                 * with no channel bounds check (src/fp_par_2d.cc:375).  The
                 * forward projection only writes channels [0, ns), so the
                 * exact adjoint gathers from those only: the range is
                 * clamped, which equals the reference wherever the pixel's
                 * footprint lies on the detector. */
                double lo = ceil(left), hi = floor(right);
                if (lo < 0) lo = 0;
                if (hi > (double)(g->ns - 1)) hi = (double)(g->ns - 1);
                double part = 0.0;
                for (double c = lo; c <= hi; c += 1.0) {
                    const unsigned is = (unsigned)c;
                    part += (1 - fabs((mid - (double)is) / step)) * pr[is];
                }
                sum += part * weights[ia];
            }
            img[(size_t)iy * g->nx + ix] = (T)sum;
        }
    }
    return 1;
}

/* Average of input rows [r0, r1) of one view and channel, in double
 * (src/helical_interpolation.cc:112-117). */
static double ORC_FN(heli_mean)(const orc_heli* h, const T* in, int view, unsigned is, int r0, int r1)
{
    double acc = 0;
    int n = 0;
    for (int r = r0; r < r1; ++r, ++n)
        acc += in[is + ((size_t)r + (size_t)view * h->nt) * h->ns];
    return acc / n;
}

/* Input sample (view, row, channel) of a 180LI corresponding ray; a view
 * outside [0, na) reads as 0 and sets *outside (the reference indexes out of
 * bounds there). */
static double ORC_FN(heli_at)(const orc_heli* h, const T* in, int view, int r, int c, int* outside)
{
    if (view < 0 || (unsigned)view >= h->na) {
        *outside = 1;
        return 0.0;
    }
    return in[(size_t)c + ((size_t)r + (size_t)view * h->nt) * h->ns];
}

/* The two-sample z interpolation of both rebinning methods
 * (src/helical_interpolation.cc:137-149); 0 when neither sample exists. */
static int ORC_FN(heli_store)(T* o, int use_cur, int use_cor, double zd, double zd2, double vcur,
                              double vcor)
{
    if (use_cur && use_cor)
        *o = (T)((zd * vcor - zd2 * vcur) / (zd - zd2));
    else if (use_cur)
        *o = (T)vcur;
    else if (use_cor)
        *o = (T)vcor;
    else
        return 0;
    return 1;
}

/* 360LI, src/helical_interpolation.cc:80-153 (helical_interpolation_360_2_,
 * the variant HelicalInterpolation360::calculate_on_cpu calls).  Views
 * [center - vpr, center + vpr) around the slice's nearest view; each output
 * view pairs the measured view with the one a rotation away on the other side
 * of the slice; each sample is the mean of the detector rows the thick slice
 * covers. */
int ORC_FN(orc_helical_360_slices)(const orc_heli* h, unsigned z0, unsigned z1, const T* in, T* out)
{
    const int vpr = (int)h->view_per_rot;
    const double center_t = (double)(h->nt - 1) / 2.0 + h->offset_t;
    const double center_s = (double)(h->ns - 1) / 2.0 + h->offset_s;
    for (unsigned iz = z0; iz < z1; ++iz) {
        const double z = heli_slice_z(h, iz);
        const int center = (int)round((z - h->couch_begin) / h->couch_mov);
        const int lo = center - vpr, hi = center + vpr - 1;
        if (lo < 0 || (unsigned)hi >= h->na) return ORC_HELI_ERR_VIEWS;
        const int first = (lo / vpr + 1) * vpr;
        T* o = out + (size_t)iz * h->view_per_rot * h->ns;
        for (int iv = 0; iv < vpr; ++iv, o += h->ns) {
            const int cur = first + iv;
            const int cor = cur >= center ? cur - vpr : cur + vpr;
            const double zd = z - h->couch_begin - cur * h->couch_mov;
            const double zd2 = z - h->couch_begin - cor * h->couch_mov;
            for (unsigned is = 0; is < h->ns; ++is) {
                const double s = ((double)is - center_s) * h->ds;
                const double cg = cos(s / h->dsd);
                int r0, r1;
                double vcur = 0, vcor = 0;
                const int ucur = heli_rows(h, center_t, zd, cg, &r0, &r1);
                if (ucur) vcur = ORC_FN(heli_mean)(h, in, cur, is, r0, r1);
                const int ucor = heli_rows(h, center_t, zd2, cg, &r0, &r1);
                if (ucor) vcor = ORC_FN(heli_mean)(h, in, cor, is, r0, r1);
                if (!ORC_FN(heli_store)(o + is, ucur, ucor, zd, zd2, vcur, vcor)) return ORC_HELI_ERR_ROWS;
            }
        }
    }
    return 1;
}

/* 180LI, src/helical_interpolation.cc:155-251 (helical_interpolation_180_2_,
 * the variant HelicalInterpolation180::calculate_on_cpu calls).  Views
 * [center - vpr/2, center - vpr/2 + vpr); the second sample of each ray is its
 * complementary ray (view offset (pi - 2 gamma) / orbit, mirrored channel),
 * bilinear in view and channel, wrapped into the view range once each way. */
int ORC_FN(orc_helical_180_slices)(const orc_heli* h, unsigned z0, unsigned z1, const T* in, T* out)
{
    const int vpr = (int)h->view_per_rot;
    const double center_t = (double)(h->nt - 1) / 2.0 + h->offset_t;
    const double center_s = (double)(h->ns - 1) / 2.0 + h->offset_s;
    int outside = 0;
    for (unsigned iz = z0; iz < z1; ++iz) {
        const double z = heli_slice_z(h, iz);
        const int center = (int)round((z - h->couch_begin) / h->couch_mov);
        const int lo = center - (int)(h->view_per_rot / 2), hi = lo + vpr - 1;
        if (lo < 0 || (unsigned)hi >= h->na) return ORC_HELI_ERR_VIEWS;
        const int first = (int)(ceil(lo / (double)h->view_per_rot) * h->view_per_rot);
        T* o = out + (size_t)iz * h->view_per_rot * h->ns;
        for (int iv = 0; iv < vpr; ++iv, o += h->ns) {
            int cur = first + iv;
            if (cur > hi) cur -= vpr;
            const double zd = z - h->couch_begin - cur * h->couch_mov;
            for (unsigned is = 0; is < h->ns; ++is) {
                const double s = ((double)is - center_s) * h->ds;
                const double gamma = s / h->dsd;
                const double cg = cos(gamma);
                int r0, r1;
                double vcur = 0, vcor = 0;
                const int ucur = heli_rows(h, center_t, zd, cg, &r0, &r1);
                if (ucur) vcur = ORC_FN(heli_mean)(h, in, cur, is, r0, r1);
                double cv = cur - (M_PI - 2 * gamma) / h->orbit;
                if (cv < lo) cv = cv + h->view_per_rot;
                if (cv > hi) cv = cv - h->view_per_rot;
                const double zd2 = z - h->couch_begin - cv * h->couch_mov;
                const int ucor = heli_rows(h, center_t, zd2, cg, &r0, &r1);
                if (ucor) {
                    const int vl = (int)floor(cv), vr = (int)ceil(cv);
                    const double u = cv - vl;
                    const double sc = center_s - s / h->ds;
                    if (sc < 0 || sc > (double)(h->ns - 1)) {
                        o[is] = (T)vcur;  /* mirrored channel off the detector */
                        continue;
                    }
                    const int cl = (int)floor(sc), cr = (int)ceil(sc);
                    const double v = sc - cl;
                    double left = 0, right = 0;
                    int n = 0;
                    for (int r = r0; r < r1; ++r, ++n) {
                        left += (1 - v) * ORC_FN(heli_at)(h, in, vl, r, cl, &outside) +
                                v * ORC_FN(heli_at)(h, in, vl, r, cr, &outside);
                        right += (1 - v) * ORC_FN(heli_at)(h, in, vr, r, cl, &outside) +
                                 v * ORC_FN(heli_at)(h, in, vr, r, cr, &outside);
                    }
                    vcor = ((1 - u) * left + u * right) / n;
                }
                if (!ORC_FN(heli_store)(o + is, ucur, ucor, zd, zd2, vcur, vcor)) return ORC_HELI_ERR_ROWS;
            }
        }
    }
    return outside ? 3 : 1;
}

#undef ORC_FN
#undef ORC_CAT
#undef ORC_CAT2

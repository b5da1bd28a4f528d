/* Test program for the reference-signature C API (include/mvkit_gb300_mv.h).
 *
 * The same source is compiled against this library (libmvkit_gb300_mv.so)
 * and against the reference's own compiled C ABI; the tests compare what
 * the two print.
 *
 *   mv_abi_probe cases <dir>
 *       a fixed table of create / params / write / read / find calls, most
 *       with a control the reference rejects; one line per call:
 *       name|status|code|operation|parameter|index|message|outputs
 *       (no call searches an image, so no GPU is needed)
 *   mv_abi_probe find <image.raw> <w> <h> <byte|uint2> <template.raw> <tw> <th>
 *       <levels|auto> <angle_start> <angle_extent> <step|auto> <metric>
 *       <tr1,tc1,tr2,tc2|-> <sr1,sc1,sr2,sc2|-> <start> <extent> <min_score>
 *       <num_matches> <max_overlap> <true|false> <highest[,lowest]> [models]
 *       mv_gen_image1 -> (mv_reduce_domain) -> mv_create_ncc_model ->
 *       mv_find_ncc_model (or mv_find_ncc_models over a tuple holding the
 *       model's handle `models` times); prints "status S" and one
 *       "match row column angle score [model]" line per match. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mvkit_gb300_mv.h"

static MvTuple td(double v) {
  MvTuple t;
  mv_create_tuple(&t, 1);
  mv_set_d(t, v, 0);
  return t;
}
static MvTuple ti(int64_t v) {
  MvTuple t;
  mv_create_tuple(&t, 1);
  mv_set_i(t, v, 0);
  return t;
}
static MvTuple ts(const char* s) {
  MvTuple t;
  MvStringView v;
  v.data = s;
  v.size = strlen(s);
  mv_create_tuple(&t, 1);
  mv_set_s(t, v, 0);
  return t;
}
static MvTuple tdd(double a, double b) {
  MvTuple t;
  mv_create_tuple(&t, 2);
  mv_set_d(t, a, 0);
  mv_set_d(t, b, 1);
  return t;
}
static MvTuple tii(int64_t a, int64_t b) {
  MvTuple t;
  mv_create_tuple(&t, 2);
  mv_set_i(t, a, 0);
  mv_set_i(t, b, 1);
  return t;
}
static MvTuple tss(const char* a, const char* b) {
  MvTuple t;
  MvStringView v;
  mv_create_tuple(&t, 2);
  v.data = a;
  v.size = strlen(a);
  mv_set_s(t, v, 0);
  v.data = b;
  v.size = strlen(b);
  mv_set_s(t, v, 1);
  return t;
}
static void drop(MvTuple t) {
  if (t) mv_destroy_tuple(t);
}

/* A tuple holding `n` handles of `model` (a model tuple of one handle). */
static MvTuple handles(MvTuple model, int n) {
  MvTuple t;
  MvHandle h;
  int i;
  mv_create_tuple(&t, (size_t)n);
  mv_get_h(model, 0, &h);
  for (i = 0; i < n; ++i) mv_set_h(t, h, (size_t)i);
  return t;
}

static void print_value(MvTuple t) {
  size_t n = 0, i;
  if (!t) {
    printf("-");
    return;
  }
  mv_length_tuple(t, &n);
  printf("[");
  for (i = 0; i < n; ++i) {
    MvValueKind k = 0;
    mv_get_type(t, i, &k);
    if (i) printf(",");
    if (k == MV_VALUE_INT64) {
      int64_t x;
      mv_get_i(t, i, &x);
      printf("%lld", (long long)x);
    } else if (k == MV_VALUE_REAL64) {
      double x;
      mv_get_d(t, i, &x);
      printf("%.17g", x);
    } else if (k == MV_VALUE_STRING) {
      MvStringView v;
      mv_get_s(t, i, &v);
      printf("\"%.*s\"", (int)v.size, v.data);
    } else if (k == MV_VALUE_HANDLE) {
      printf("handle");
    } else {
      printf("empty");
    }
  }
  printf("]");
}

static void report(const char* name, MvStatus st, MvTuple* outs, int nout) {
  MvErrorInfo e;
  int i;
  memset(&e, 0, sizeof(e));
  mv_get_last_error_info(&e);
  if (st == MV_STATUS_OK)
    printf("%s|0|||||", name);
  else
    printf("%s|%d|%d|%.*s|%.*s|%lld|%.*s", name, st, e.code, (int)e.operation.size,
           e.operation.data ? e.operation.data : "", (int)e.parameter.size, e.parameter.data ? e.parameter.data : "",
           (long long)e.parameter_index, (int)e.message.size, e.message.data ? e.message.data : "");
  printf("|");
  for (i = 0; i < nout; ++i) {
    if (i) printf(" ");
    print_value(st == MV_STATUS_OK ? outs[i] : NULL);
  }
  printf("\n");
  for (i = 0; i < nout; ++i) {
    if (st == MV_STATUS_OK) drop(outs[i]);
    outs[i] = NULL;
  }
}

/* A textured test template (integer arithmetic only). */
static void pattern(unsigned char* p, int w, int h, int seed) {
  int r, c;
  for (r = 0; r < h; ++r)
    for (c = 0; c < w; ++c) {
      unsigned v = (unsigned)(r * 37 + c * 11 + seed * 101) ^ (unsigned)((r / 5) * (c / 7) * 29 + seed);
      p[r * w + c] = (unsigned char)(40 + (v * 2654435761u >> 24) % 180);
    }
}

static MvObject image(const char* type, int w, int h, const void* px) {
  MvObject o = NULL;
  MvTuple t = ts(type), tw = ti(w), th = ti(h), tp = ti((int64_t)(size_t)px);
  mv_gen_image1(&o, t, tw, th, tp);
  drop(t);
  drop(tw);
  drop(th);
  drop(tp);
  return o;
}

static MvObject reduced(MvObject im, int r1, int c1, int r2, int c2) {
  MvObject rect = NULL, out = NULL;
  MvTuple a = ti(r1), b = ti(c1), c = ti(r2), d = ti(c2);
  mv_gen_rectangle1(&rect, a, b, c, d);
  mv_reduce_domain(im, rect, &out);
  mv_clear_obj(rect);
  drop(a);
  drop(b);
  drop(c);
  drop(d);
  return out;
}

/* find with every control given; outs: row, column, angle, score */
static MvStatus find(MvObject im, MvTuple model, MvTuple a0, MvTuple ext, MvTuple score, MvTuple nm, MvTuple ov,
                     MvTuple sp, MvTuple lv, MvTuple* outs) {
  return mv_find_ncc_model(im, model, a0, ext, score, nm, ov, sp, lv, &outs[0], &outs[1], &outs[2], &outs[3]);
}

static int run_cases(const char* dir) {
  static unsigned char tpl[64 * 64], tpl2[96 * 80];
  static unsigned short tpl16[64 * 64];
  MvTuple outs[5] = {NULL, NULL, NULL, NULL, NULL};
  MvTuple model = NULL, model2 = NULL, cleared = NULL, mt;
  MvObject t8, t16, empty = NULL, timg, region = NULL, roi, real = NULL;
  MvStatus st;
  char path[4096];
  int i;
  /* controls reused below */
  MvTuple l3 = ti(3), zero = td(0), half = td(0.5), au = ts("auto"), pol = ts("use_polarity");
  MvTuple s7 = td(0.7), one = ti(1), ov = td(0.5), tru = ts("true"), lv0 = ti(0);

  pattern(tpl, 64, 64, 1);
  pattern(tpl2, 96, 80, 2);
  for (i = 0; i < 64 * 64; ++i) tpl16[i] = (unsigned short)(tpl[i] * 13 + (i % 7));
  t8 = image("byte", 64, 64, tpl);
  t16 = image("uint2", 64, 64, tpl16);
  timg = image("byte", 96, 80, tpl2);
  mv_gen_empty_obj(&empty);
  {
    MvTuple a = ti(2), b = ti(3), c = ti(20), d = ti(30);
    mv_gen_rectangle1(&region, a, b, c, d);
    drop(a);
    drop(b);
    drop(c);
    drop(d);
  }
  roi = reduced(timg, 8, 10, 70, 85);
  {
    MvTuple a = ts("real"), b = ti(32), c = ti(32);
    mv_gen_image_const(&real, a, b, c);
    drop(a);
    drop(b);
    drop(c);
  }

  /* ---------------------------------------------------------- create */
  st = mv_create_ncc_model(t8, l3, zero, half, au, pol, &model);
  report("create_ok", st, outs, 0);
  st = mv_get_ncc_model_params(model, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
  report("params_ok", st, outs, 5);
  {
    MvTuple lvl = ts("auto");
    st = mv_create_ncc_model(t8, lvl, zero, half, au, pol, &mt);
    report("create_levels_auto", st, outs, 0);
    if (st == 0) {
      st = mv_get_ncc_model_params(mt, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
      report("params_levels_auto", st, outs, 5);
      drop(mt);
    }
    drop(lvl);
  }
#define CREATE(name, tmpl, lv, a0, ext, step, metric)                                         \
  do {                                                                                        \
    MvTuple m_ = NULL;                                                                        \
    st = mv_create_ncc_model(tmpl, lv, a0, ext, step, metric, &m_);                           \
    report(name, st, outs, 0);                                                                \
    if (st == 0) {                                                                            \
      st = mv_get_ncc_model_params(m_, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);     \
      report(name "_params", st, outs, 5);                                                    \
      drop(m_);                                                                               \
    }                                                                                         \
  } while (0)
  {
    MvTuple many = ts("many"), l17 = ti(17), lreal = td(3.0), lpair = tii(3, 4), big = td(0.5), sz = td(0.0),
            bad = ts("use_polarityx"), mint = ti(3), two = tss("use_polarity", "use_polarity"), inf = td(INFINITY),
            ign = ts("ignore_global_polarity"), l16 = ti(16), neg = ti(-1), ext2 = td(6.2831853071795862),
            step = td(0.05);
    CREATE("create_levels_many", t8, many, zero, half, au, pol);
    CREATE("create_levels_17", t8, l17, zero, half, au, pol);
    CREATE("create_levels_neg", t8, neg, zero, half, au, pol);
    CREATE("create_levels_real", t8, lreal, zero, half, au, pol);
    CREATE("create_levels_pair", t8, lpair, zero, half, au, pol);
    CREATE("create_step_big", t8, l3, zero, half, big, pol);
    CREATE("create_step_zero", t8, l3, zero, half, sz, pol);
    CREATE("create_step_explicit", t8, l3, zero, half, step, pol);
    CREATE("create_metric_bad", t8, l3, zero, half, au, bad);
    CREATE("create_metric_int", t8, l3, zero, half, au, mint);
    CREATE("create_metric_two", t8, l3, zero, half, au, two);
    CREATE("create_metric_ignore", t8, l3, zero, half, au, ign);
    CREATE("create_start_inf", t8, l3, inf, half, au, pol);
    CREATE("create_start_null", t8, l3, NULL, half, au, pol);
    CREATE("create_extent_full", t8, l3, zero, ext2, au, pol);
    CREATE("create_null_template", NULL, l3, zero, half, au, pol);
    CREATE("create_empty_template", empty, l3, zero, half, au, pol);
    CREATE("create_real_template", real, l3, zero, half, au, pol);
    CREATE("create_region_template", region, l3, zero, half, au, pol);
    CREATE("create_roi_template", roi, l3, zero, half, au, pol);
    CREATE("create_u16", t16, l3, zero, half, au, pol);
    CREATE("create_levels_16", t8, l16, zero, half, au, pol);
    st = mv_create_ncc_model(t8, l3, zero, half, au, pol, NULL);
    report("create_null_output", st, outs, 0);
    drop(many);
    drop(l17);
    drop(lreal);
    drop(lpair);
    drop(big);
    drop(sz);
    drop(bad);
    drop(mint);
    drop(two);
    drop(inf);
    drop(ign);
    drop(l16);
    drop(neg);
    drop(ext2);
    drop(step);
  }

  /* ---------------------------------------------------------- params */
  st = mv_get_ncc_model_params(NULL, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
  report("params_null_model", st, outs, 5);
  st = mv_get_ncc_model_params(half, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
  report("params_not_handle", st, outs, 5);
  mv_create_ncc_model(t8, l3, zero, half, au, pol, &cleared);
  st = mv_clear_handle(cleared);
  report("clear_handle", st, outs, 0);
  st = mv_get_ncc_model_params(cleared, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
  report("params_cleared", st, outs, 5);
  st = mv_clear_handle(half);
  report("clear_handle_not_handle", st, outs, 0);

  /* ------------------------------------------------------ write / read */
  {
    MvTuple name, bad = ts(""), missing = ts("/nonexistent-dir/x.ncm"), junk;
    FILE* f;
    snprintf(path, sizeof(path), "%s/model.ncm", dir);
    name = ts(path);
    st = mv_write_ncc_model(model, name);
    report("write_ok", st, outs, 0);
    st = mv_read_ncc_model(name, &model2);
    report("read_ok", st, outs, 0);
    if (st == 0) {
      st = mv_get_ncc_model_params(model2, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
      report("params_read", st, outs, 5);
    }
    st = mv_write_ncc_model(model, bad);
    report("write_empty_name", st, outs, 0);
    st = mv_write_ncc_model(half, name);
    report("write_not_handle", st, outs, 0);
    st = mv_read_ncc_model(missing, &mt);
    report("read_missing", st, outs, 0);
    snprintf(path, sizeof(path), "%s/junk.ncm", dir);
    f = fopen(path, "wb");
    if (f) {
      fputs("MVKIT_NCC 1\nnot a model\n", f);
      fclose(f);
    }
    junk = ts(path);
    st = mv_read_ncc_model(junk, &mt);
    report("read_junk", st, outs, 0);
    st = mv_read_ncc_model(name, NULL);
    report("read_null_output", st, outs, 0);
    drop(name);
    drop(bad);
    drop(missing);
    drop(junk);
  }

  /* ------------------------------------------------------------- find */
  st = find(empty, model, zero, half, s7, one, ov, tru, lv0, outs);
  report("find_empty_image", st, outs, 4);
#define FIND(name, im, m, a0, ext, sc, nm, o, sp, lv)          \
  do {                                                        \
    st = find(im, m, a0, ext, sc, nm, o, sp, lv, outs);       \
    report(name, st, outs, 4);                                \
  } while (0)
  {
    MvTuple sbig = td(1.5), sneg = td(-0.1), e7 = td(7.0), en = td(-0.1), mneg = ti(-1), mreal = td(1.0),
            spb = ti(1), spy = ts("yes"), l3v, lneg = ti(-1), lpz = tii(3, 0), lp = tii(3, 2), s2 = tdd(0.5, 0.6),
            two = handles(model, 2), one_h = handles(model, 1), ovb = td(2.0), nanv = td(NAN), spf = ts("false"),
            estr = ts("wide");
    mv_create_tuple(&l3v, 3);
    for (i = 0; i < 3; ++i) mv_set_i(l3v, 3, (size_t)i);
    FIND("find_score_big", empty, model, zero, half, sbig, one, ov, tru, lv0);
    FIND("find_score_neg", empty, model, zero, half, sneg, one, ov, tru, lv0);
    FIND("find_score_nan", empty, model, zero, half, nanv, one, ov, tru, lv0);
    FIND("find_extent_7", empty, model, zero, e7, s7, one, ov, tru, lv0);
    FIND("find_extent_neg", empty, model, zero, en, s7, one, ov, tru, lv0);
    FIND("find_extent_string", empty, model, zero, estr, s7, one, ov, tru, lv0);
    FIND("find_overlap_2", empty, model, zero, half, s7, one, ovb, tru, lv0);
    FIND("find_matches_neg", empty, model, zero, half, s7, mneg, ov, tru, lv0);
    FIND("find_matches_real", empty, model, zero, half, s7, mreal, ov, tru, lv0);
    FIND("find_subpixel_int", empty, model, zero, half, s7, one, ov, spb, lv0);
    FIND("find_subpixel_yes", empty, model, zero, half, s7, one, ov, spy, lv0);
    FIND("find_subpixel_false", empty, model, zero, half, s7, one, ov, spf, lv0);
    FIND("find_levels_three", empty, model, zero, half, s7, one, ov, tru, l3v);
    FIND("find_levels_neg", empty, model, zero, half, s7, one, ov, tru, lneg);
    FIND("find_levels_pair_zero", empty, model, zero, half, s7, one, ov, tru, lpz);
    FIND("find_levels_pair", empty, model, zero, half, s7, one, ov, tru, lp);
    FIND("find_two_scores", empty, model, zero, half, s2, one, ov, tru, lv0);
    FIND("find_two_models", empty, two, zero, half, s7, one, ov, tru, lv0);
    FIND("find_handle_tuple", empty, one_h, zero, half, s7, one, ov, tru, lv0);
    FIND("find_model_not_handle", empty, half, zero, half, s7, one, ov, tru, lv0);
    FIND("find_model_cleared", empty, cleared, zero, half, s7, one, ov, tru, lv0);
    FIND("find_model_null", empty, NULL, zero, half, s7, one, ov, tru, lv0);
    FIND("find_start_null", empty, model, NULL, half, s7, one, ov, tru, lv0);
    FIND("find_null_image", NULL, model, zero, half, s7, one, ov, tru, lv0);
    FIND("find_region_image", region, model, zero, half, s7, one, ov, tru, lv0);
    FIND("find_real_image", real, model, zero, half, s7, one, ov, tru, lv0);
    st = mv_find_ncc_model(empty, model, zero, half, s7, one, ov, tru, lv0, NULL, &outs[1], &outs[2], &outs[3]);
    report("find_null_row", st, outs, 4);
    st = mv_find_ncc_model(empty, model, zero, half, s7, one, ov, tru, lv0, &outs[0], &outs[0], &outs[2], &outs[3]);
    report("find_same_outputs", st, outs, 4);

    /* FindNccModels */
    st = mv_find_ncc_models(empty, two, zero, half, s7, one, ov, tru, lv0, &outs[0], &outs[1], &outs[2], &outs[3],
                            &outs[4]);
    report("models_empty_image", st, outs, 5);
    {
      MvTuple sbad = tdd(0.5, 1.5), l4, s3;
      mv_create_tuple(&l4, 4);
      for (i = 0; i < 4; ++i) mv_set_i(l4, (i % 2) ? 1 : 3, (size_t)i);
      mv_create_tuple(&s3, 3);
      for (i = 0; i < 3; ++i) mv_set_d(s3, 0.5, (size_t)i);
      st = mv_find_ncc_models(empty, two, zero, half, sbad, one, ov, tru, lv0, &outs[0], &outs[1], &outs[2],
                              &outs[3], &outs[4]);
      report("models_score_per_model_bad", st, outs, 5);
      st = mv_find_ncc_models(empty, two, zero, half, s7, one, ov, tru, l4, &outs[0], &outs[1], &outs[2], &outs[3],
                              &outs[4]);
      report("models_level_pairs", st, outs, 5);
      st = mv_find_ncc_models(empty, two, zero, half, s3, one, ov, tru, lv0, &outs[0], &outs[1], &outs[2], &outs[3],
                              &outs[4]);
      report("models_three_scores", st, outs, 5);
      st = mv_find_ncc_models(empty, NULL, zero, half, s7, one, ov, tru, lv0, &outs[0], &outs[1], &outs[2], &outs[3],
                              &outs[4]);
      report("models_no_model", st, outs, 5);
      drop(sbad);
      drop(l4);
      drop(s3);
    }
    drop(sbig);
    drop(sneg);
    drop(e7);
    drop(en);
    drop(mneg);
    drop(mreal);
    drop(spb);
    drop(spy);
    drop(l3v);
    drop(lneg);
    drop(lpz);
    drop(lp);
    drop(s2);
    drop(two);
    drop(one_h);
    drop(ovb);
    drop(nanv);
    drop(spf);
    drop(estr);
  }
  /* tuple and region layer */
  {
    MvTuple rr = NULL, rb = NULL, re = NULL, cnt = NULL;
    MvObject dom = NULL;
    outs[0] = outs[1] = outs[2] = NULL;
    st = mv_get_region_runs(region, &outs[0], &outs[1], &outs[2]);
    report("region_runs", st, outs, 3);
    st = mv_get_domain(roi, &dom);
    report("get_domain", st, outs, 0);
    if (st == 0) {
      st = mv_get_region_runs(dom, &rr, &rb, &re);
      outs[0] = rr;
      outs[1] = rb;
      outs[2] = re;
      report("domain_runs", st, outs, 3);
      mv_clear_obj(dom);
    }
    st = mv_count_obj(empty, &cnt);
    outs[0] = cnt;
    report("count_empty", st, outs, 1);
  }
  drop(model);
  drop(model2);
  drop(cleared);
  drop(l3);
  drop(zero);
  drop(half);
  drop(au);
  drop(pol);
  drop(s7);
  drop(one);
  drop(ov);
  drop(tru);
  drop(lv0);
  mv_clear_obj(t8);
  mv_clear_obj(t16);
  mv_clear_obj(timg);
  mv_clear_obj(empty);
  mv_clear_obj(region);
  mv_clear_obj(roi);
  mv_clear_obj(real);
  return 0;
}

static void* read_raw(const char* path, size_t bytes) {
  FILE* f = fopen(path, "rb");
  void* p = malloc(bytes ? bytes : 1);
  if (!f || !p || fread(p, 1, bytes, f) != bytes) {
    fprintf(stderr, "cannot read %s\n", path);
    exit(2);
  }
  fclose(f);
  return p;
}

static MvTuple number_or_auto(const char* s) {
  return strcmp(s, "auto") == 0 ? ts("auto") : (strchr(s, '.') ? td(atof(s)) : ti(atoll(s)));
}

static MvObject with_roi(MvObject im, const char* spec) {
  int r1, c1, r2, c2;
  MvObject out;
  if (strcmp(spec, "-") == 0 || sscanf(spec, "%d,%d,%d,%d", &r1, &c1, &r2, &c2) != 4) return im;
  out = reduced(im, r1, c1, r2, c2);
  mv_clear_obj(im);
  return out;
}

static int run_find(int argc, char** argv) {
  int w, h, tw, th, k, models = 0, hi = 0, lo = -1;
  size_t bpp, n = 0, i;
  void *px, *tp;
  MvObject im, tm;
  MvTuple model = NULL, outs[5] = {NULL, NULL, NULL, NULL, NULL}, lv, a0, ext, sc, nm, ov, sp, ids;
  MvStatus st;
  if (argc < 22) {
    fprintf(stderr, "usage: see the file header\n");
    return 2;
  }
  w = atoi(argv[3]);
  h = atoi(argv[4]);
  bpp = strcmp(argv[5], "uint2") == 0 ? 2 : 1;
  tw = atoi(argv[7]);
  th = atoi(argv[8]);
  px = read_raw(argv[2], (size_t)w * (size_t)h * bpp);
  tp = read_raw(argv[6], (size_t)tw * (size_t)th * bpp);
  im = with_roi(image(argv[5], w, h, px), argv[15]);
  tm = with_roi(image(argv[5], tw, th, tp), argv[14]);
  {
    MvTuple l = number_or_auto(argv[9]), s = td(atof(argv[10])), e = td(atof(argv[11])), stp = number_or_auto(argv[12]),
            m = ts(argv[13]);
    st = mv_create_ncc_model(tm, l, s, e, stp, m, &model);
    drop(l);
    drop(s);
    drop(e);
    drop(stp);
    drop(m);
  }
  if (st != MV_STATUS_OK) {
    MvStringView v;
    mv_get_last_error(&v);
    printf("status %d\nerror %.*s\n", st, (int)v.size, v.data);
    return 0;
  }
  a0 = td(atof(argv[16]));
  ext = td(atof(argv[17]));
  sc = td(atof(argv[18]));
  nm = ti(atoll(argv[19]));
  ov = td(atof(argv[20]));
  sp = ts(argv[21]);
  if (sscanf(argv[22], "%d,%d", &hi, &lo) == 2)
    lv = tii(hi, lo);
  else
    lv = ti(atoi(argv[22]));
  if (argc > 23) models = atoi(argv[23]);
  if (models > 0) {
    ids = handles(model, models);
    st = mv_find_ncc_models(im, ids, a0, ext, sc, nm, ov, sp, lv, &outs[0], &outs[1], &outs[2], &outs[3], &outs[4]);
    drop(ids);
  } else {
    st = mv_find_ncc_model(im, model, a0, ext, sc, nm, ov, sp, lv, &outs[0], &outs[1], &outs[2], &outs[3]);
  }
  printf("status %d\n", st);
  if (st != MV_STATUS_OK) {
    MvStringView v;
    mv_get_last_error(&v);
    printf("error %.*s\n", (int)v.size, v.data);
  } else {
    mv_length_tuple(outs[0], &n);
    for (i = 0; i < n; ++i) {
      double v[4];
      for (k = 0; k < 4; ++k) mv_get_d(outs[k], i, &v[k]);
      printf("match %.17g %.17g %.17g %.17g", v[0], v[1], v[2], v[3]);
      if (models > 0) {
        int64_t mi;
        mv_get_i(outs[4], i, &mi);
        printf(" %lld", (long long)mi);
      }
      printf("\n");
    }
    for (k = 0; k < 5; ++k) drop(outs[k]);
  }
  drop(model);
  drop(a0);
  drop(ext);
  drop(sc);
  drop(nm);
  drop(ov);
  drop(sp);
  drop(lv);
  mv_clear_obj(im);
  mv_clear_obj(tm);
  free(px);
  free(tp);
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 3 && strcmp(argv[1], "cases") == 0) return run_cases(argv[2]);
  if (argc >= 2 && strcmp(argv[1], "find") == 0) return run_find(argc, argv);
  fprintf(stderr, "usage: mv_abi_probe cases <dir> | find ...\n");
  return 2;
}

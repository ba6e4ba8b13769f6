// Text result files of a single-component run: GSOutput::writeResults
// (reference src/solve/result_writer.cpp:64-430) for one genetic component
// (GA for GBLUP, HA for ssGBLUP, PA for pedigree BLUP) without the ANOVA table.
//
//  * <prefix>.vars: "Item\tVar\tVar_SE\th2\th2_SE\th2_Pr(Chisq)", the component
//    row and the "e" row (:117-197).  h2 = var_k / (sum var + var_e); its SE by
//    the delta method over the components' SEs; Pr = erfc(|h2 / se| / sqrt 2)
//    (two-sided normal), "<2e-16" below 2e-16, 1 when se < 1e-12 (:21-31).
//  * <prefix>.beta: "Levels\tEstimation\tSE", one row per fixed-effect column,
//    SE "nan" when not computed (:199-236).
//  * <prefix>.rand: "ID\t<tag>\tresiduals\tn_obs".  Per animal the mean of its
//    records' random-effect values and residuals y - Xb - u and its record
//    count; animals in order of first record, then the animals without records
//    sorted by ID, whose value is their solution (:302-430).
// Numbers are written with the default C++ stream format (6 significant
// digits), as the reference's ofstream does.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <limits>
#include <sstream>
#include <string>
#include <vector>
#include "handle.h"

namespace {

std::string fmt(double v) {
  std::ostringstream s;
  s << v;
  return s.str();
}

std::string pval_str(double val, double se) {
  const double p = se < 1e-12 ? 1.0 : std::erfc((val / se) / std::sqrt(2.0));
  return p < 2e-16 ? std::string("<2e-16") : fmt(p);
}

std::ofstream open_out(const char* path) {
  CBX_REQUIRE(path && *path, CBX_ERR_ARG, "empty output path");
  std::ofstream f(path);
  CBX_REQUIRE(f.good(), CBX_ERR_ARG, std::string("cannot open ") + path);
  return f;
}

}  // namespace

extern "C" int cbx_write_vars(const char* path, const char* tag, double var_u, double se_u, double var_e,
                              double se_e) {
  try {
    std::ofstream f = open_out(path);
    const std::string t = (tag && *tag) ? tag : "GA";
    const double total = var_e + var_u;
    f << "Item\tVar\tVar_SE\th2\th2_SE\th2_Pr(Chisq)\n";
    {
      const double h2 = total > 1e-9 ? var_u / total : 0.0;
      const double den = total * total;
      const double dh_du = (total - var_u) / den, dh_de = -var_u / den;
      const double v = dh_du * dh_du * se_u * se_u + dh_de * dh_de * se_e * se_e;
      const double se_h2 = std::sqrt(std::max(0.0, v));
      f << t << "\t" << fmt(var_u) << "\t" << fmt(se_u) << "\t" << fmt(h2) << "\t" << fmt(se_h2) << "\t"
        << pval_str(h2, se_h2) << "\n";
    }
    {
      const double h2e = total > 1e-9 ? var_e / total : 0.0;
      const double den = total * total;
      const double d_e = (total - var_e) / den, d_o = -var_e / den;
      const double v = d_e * d_e * se_e * se_e + d_o * d_o * se_u * se_u;
      const double se_h2e = std::sqrt(std::max(0.0, v));
      f << "e\t" << fmt(var_e) << "\t" << fmt(se_e) << "\t" << fmt(h2e) << "\t" << fmt(se_h2e) << "\t"
        << pval_str(h2e, se_h2e) << "\n";
    }
    CBX_REQUIRE(f.good(), CBX_ERR_ARG, std::string("write failed: ") + path);
    return CBX_OK;
  } catch (const cbx::Error& e) {
    return e.code;
  } catch (...) {
    return CBX_ERR_ARG;
  }
}

extern "C" int cbx_write_beta(const char* path, int64_t p, const char* const* names, const double* beta,
                              const double* beta_se) {
  try {
    CBX_REQUIRE(p >= 0 && names && beta, CBX_ERR_ARG, "bad fixed-effect arrays");
    std::ofstream f = open_out(path);
    f << "Levels\tEstimation\tSE\n";
    for (int64_t i = 0; i < p; ++i) {
      f << (names[i] ? names[i] : "") << "\t" << fmt(beta[i]);
      if (beta_se) f << "\t" << fmt(beta_se[i]);
      else f << "\tnan";
      f << "\n";
    }
    CBX_REQUIRE(f.good(), CBX_ERR_ARG, std::string("write failed: ") + path);
    return CBX_OK;
  } catch (const cbx::Error& e) {
    return e.code;
  } catch (...) {
    return CBX_ERR_ARG;
  }
}

extern "C" int cbx_write_rand(const char* path, const char* tag, int64_t n_rec, const double* y,
                              const int32_t* aid, const int64_t* fx_ptr, const int32_t* fx_col,
                              const double* fx_val, int64_t p, const double* beta, int64_t q, const double* u,
                              const char* const* ids) {
  try {
    CBX_REQUIRE(n_rec >= 0 && q >= 0 && p >= 0, CBX_ERR_ARG, "bad sizes");
    CBX_REQUIRE((n_rec == 0 || (y && aid && fx_ptr)) && (q == 0 || u) && (p == 0 || beta), CBX_ERR_ARG,
                "null arrays");
    std::ofstream f = open_out(path);
    const std::string t = (tag && *tag) ? tag : "GA";
    f << "ID\t" << t << "\tresiduals\tn_obs\n";
    std::vector<double> usum(q, 0.0), rsum(q, 0.0);
    std::vector<int64_t> cnt(q, 0);
    std::vector<int64_t> order;
    order.reserve(q);
    std::vector<char> seen(q, 0);
    for (int64_t i = 0; i < n_rec; ++i) {
      double xb = 0.0;
      for (int64_t a = fx_ptr[i]; a < fx_ptr[i + 1]; ++a)
        if (fx_col[a] >= 0 && fx_col[a] < p) xb += fx_val[a] * beta[fx_col[a]];
      const int64_t k = (int64_t)aid[i] - 1;
      const double uv = (k >= 0 && k < q) ? u[k] : 0.0;
      const double res = y[i] - (xb + uv);
      if (k >= 0 && k < q) {
        rsum[k] += res;
        usum[k] += uv;
        cnt[k] += 1;
        if (!seen[k]) {
          seen[k] = 1;
          order.push_back(k);
        }
      }
    }
    auto id_of = [&](int64_t k) {
      const char* s = ids ? ids[k] : nullptr;
      return (s && *s) ? std::string(s) : "UNK_" + std::to_string(k + 1);
    };
    std::vector<int64_t> rest;
    for (int64_t k = 0; k < q; ++k)
      if (!seen[k]) rest.push_back(k);
    std::sort(rest.begin(), rest.end(), [&](int64_t a, int64_t b) {
      const std::string sa = ids && ids[a] ? ids[a] : "", sb = ids && ids[b] ? ids[b] : "";
      return sa < sb;
    });
    order.insert(order.end(), rest.begin(), rest.end());
    for (int64_t k : order) {
      f << id_of(k);
      if (cnt[k] > 0) f << "\t" << fmt(usum[k] / (double)cnt[k]);
      else f << "\t" << fmt(u[k]);
      if (cnt[k] > 0) f << "\t" << fmt(rsum[k] / (double)cnt[k]);
      else f << "\tnan";
      f << "\t" << cnt[k] << "\n";
    }
    CBX_REQUIRE(f.good(), CBX_ERR_ARG, std::string("write failed: ") + path);
    return CBX_OK;
  } catch (const cbx::Error& e) {
    return e.code;
  } catch (...) {
    return CBX_ERR_ARG;
  }
}

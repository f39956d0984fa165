// Coverage ingest: the reference's .vis text reader and its visibility
// weighting (uniform / robust by a gridded histogram), the steps that produce
// the u, v, w and weights an operator is built from.
#pragma once
#include <complex>
#include <cstdint>
#include <string>

namespace pg {

// Rows (lines) of a .vis file (utilities.cc:148-153).
int64_t vis_file_rows(const std::string &path);

// utilities::read_visibility (utilities.cc:140-188): per row u v [w] re im
// sigma, separated by white space; v is negated (utilities.cc:178) and the
// weight is 1 / sigma.  w may be null when !w_term (it is then left alone).
void read_visibility(const std::string &path, bool w_term, int64_t rows, double *u, double *v,
                     double *w, std::complex<double> *vis, std::complex<double> *weights);

enum Weighting : int { kWeightNone = 0, kWeightNatural = 1, kWeightWhiten = 2,
                       kWeightUniform = 3, kWeightRobust = 4 };

// utilities::init_weights (utilities.cc:569-608).  The uniform and robust
// histograms and reductions run on `device`; host buffers in and out.
void init_weights(const double *u, const double *v, const std::complex<double> *weights,
                  int64_t M, double oversample_factor, int weighting, double R, int ftsizeu,
                  int ftsizev, int device, std::complex<double> *out);

}  // namespace pg

// Host side of the drop-in: the parameter file, the output files and the run
// loop of the reference's standard path, driving the GPU through include/axs.h.
#pragma once

#include <cstdio>
#include <string>

#include "axs.h"

namespace axs_host {

constexpr int kMaxLen = 200;   // MAX_LEN of src/common/common.hpp:25

// The reference's `struct parameters` (src/common/common.hpp:30-69), with the
// same member names and types, plus the GPU-path options (all optional in the
// parameter file, see axs_params.cpp).
struct RunConfig {
    // physics / lattice (reference tags)
    float lambda = 0;
    int enable_PRS = 0;
    float T_initial = 0;
    int NDIMS = 0;
    int N = 0;
    float space_step = 0;
    float time_step = 0;
    int stencil_setting = 0;
    unsigned int seed = 0;
    // output (reference tags)
    int write_output_file = 0;
    char output_file_path[kMaxLen] = {0};
    int save_snapshots = 0;
    int n_snapshots = 0;
    char output_directory[kMaxLen] = {0};
    int save_fields = 0;
    int save_strings = 0;
    int save_pk = 0;
    int sample_time_series = 0;
    int n_samples = 0;
    char ts_output_path[kMaxLen] = {0};
    int sample_strings = 0;
    int sample_background = 0;
    int thr = 0;
    int enable_amr = 0;
    float refinement_threshold = 0;
    int init_from_snapshot = 0;
    float tau_initial = 0;
    // GPU-path options (new, optional)
    int gpu_precision = 64;        // 32 or 64
    int gpu_prs = 1;               // potential coefficient lambda / tau^(2 prs); 1 = reference
    int gpu_form = 0;              // 0 = vvsl_field_rescaled (reference), 1 = vvsl_hamiltonian_form
    int gpu_laplacian = 0;         // 0 = stencil (reference default), 1 = compute_laplacian_fft
    int init_mode = 0;             // 0 = gaussian_thermal (reference), 1 = flat k_cut
    float k_cut = 1.0f;            // flat init cut-off (physical k)
    int string_interval = 0;       // > 0: also find strings every this many steps
    int spectrum_interval = 0;     // > 0: axion kinetic spectrum every this many steps
    int spectrum_bins = 128;
    int final_step = 0;            // > 0 overrides the light-crossing final step
    int check_finite = 0;          // 1: NaN/Inf check at every output step
    char gpu_restart_file[kMaxLen] = {0};     // start from this axs_checkpoint file instead of
                                              // gaussian_thermal; the run continues at its step
    char gpu_checkpoint_file[kMaxLen] = {0};  // write an axs_checkpoint file after the last step
};

// read_parameter_file (src/common/read_parameters.cpp:182-238): every
// reference tag must appear exactly once; GPU tags at most once. On error
// returns AXS_ERR_PARSE and the reference's message in `err`.
int read_parameter_file(const char *fname, RunConfig &c, std::string &err);

axs_params to_params(const RunConfig &c);

// Output streams and writers of src/common/fileio.cpp.
struct Output {
    FILE *main = stdout;
    FILE *time_series = nullptr;
    FILE *snapshot_timings = nullptr;
    std::string dir;
};
int open_outputs(const RunConfig &c, Output &o, std::string &err);
void close_outputs(const RunConfig &c, Output &o);
void save_field_data(Output &o, const char *name, const double *data, long long n);
void save_strings(Output &o, const char *name, const int *pos, long long n, int ndims);
void save_pk(Output &o, const char *name, const double *pk, const double *ks, const int *count, int nbins);
void save_axion_spectrum(Output &o, const char *name, const double *k, const double *pk, const long long *count, int nbins);

// run_standard (src/standard/s_run.cpp:26-232) on the GPU.
int run_standard(const RunConfig &c, Output &o, std::string &err);

}  // namespace axs_host

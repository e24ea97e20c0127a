// Parameter-file reader with the reference's rules
// (src/common/read_parameters.cpp:182-238, default.param): lines whose first
// token is a tag and second a value; '%' starts a comment line; a tag that is
// unknown or given twice is an error; every reference tag is required. The
// GPU-path tags are optional, so the reference's own default.param reads as is.
#include <cstdlib>
#include <cstring>
#include <vector>

#include "axs_host.h"

namespace axs_host {

namespace {
enum Type { FLOAT, INT, UINT, STRING };
struct Tag {
    const char *name;
    Type type;
    void *addr;
    bool required;
    bool seen;
};
}  // namespace

int read_parameter_file(const char *fname, RunConfig &c, std::string &err) {
    std::vector<Tag> tags = {
        {"lambda", FLOAT, &c.lambda, true, false},
        {"enable_PRS", INT, &c.enable_PRS, true, false},
        {"T_initial", FLOAT, &c.T_initial, true, false},
        {"NDIMS", INT, &c.NDIMS, true, false},
        {"N", INT, &c.N, true, false},
        {"space_step", FLOAT, &c.space_step, true, false},
        {"time_step", FLOAT, &c.time_step, true, false},
        {"stencil_setting", INT, &c.stencil_setting, true, false},
        {"seed", UINT, &c.seed, true, false},
        {"write_output_file", INT, &c.write_output_file, true, false},
        {"output_file_path", STRING, c.output_file_path, true, false},
        {"save_snapshots", INT, &c.save_snapshots, true, false},
        {"n_snapshots", INT, &c.n_snapshots, true, false},
        {"output_directory", STRING, c.output_directory, true, false},
        {"save_fields", INT, &c.save_fields, true, false},
        {"save_strings", INT, &c.save_strings, true, false},
        {"save_pk", INT, &c.save_pk, true, false},
        {"sample_time_series", INT, &c.sample_time_series, true, false},
        {"n_samples", INT, &c.n_samples, true, false},
        {"ts_output_path", STRING, c.ts_output_path, true, false},
        {"sample_strings", INT, &c.sample_strings, true, false},
        {"sample_background", INT, &c.sample_background, true, false},
        {"thr", INT, &c.thr, true, false},
        {"enable_amr", INT, &c.enable_amr, true, false},
        {"init_from_snapshot", INT, &c.init_from_snapshot, true, false},
        {"tau_initial", FLOAT, &c.tau_initial, true, false},
        {"refinement_threshold", FLOAT, &c.refinement_threshold, true, false},
        {"gpu_precision", INT, &c.gpu_precision, false, false},
        {"gpu_prs", INT, &c.gpu_prs, false, false},
        {"gpu_form", INT, &c.gpu_form, false, false},
        {"gpu_laplacian", INT, &c.gpu_laplacian, false, false},
        {"init_mode", INT, &c.init_mode, false, false},
        {"k_cut", FLOAT, &c.k_cut, false, false},
        {"string_interval", INT, &c.string_interval, false, false},
        {"spectrum_interval", INT, &c.spectrum_interval, false, false},
        {"spectrum_bins", INT, &c.spectrum_bins, false, false},
        {"final_step", INT, &c.final_step, false, false},
        {"check_finite", INT, &c.check_finite, false, false},
        {"gpu_restart_file", STRING, c.gpu_restart_file, false, false},
        {"gpu_checkpoint_file", STRING, c.gpu_checkpoint_file, false, false},
    };
    FILE *fd = fopen(fname, "r");
    if (!fd) {
        err = std::string("Error: cannot open parameter file ") + fname;
        return AXS_ERR_PARSE;
    }
    char line[kMaxLen], b1[kMaxLen], b2[kMaxLen], b3[kMaxLen];
    while (fgets(line, sizeof line, fd)) {
        if (sscanf(line, "%199s%199s%199s", b1, b2, b3) < 2 || b1[0] == '%') continue;
        Tag *t = nullptr;
        for (Tag &x : tags)
            if (!x.seen && strcmp(b1, x.name) == 0) { t = &x; break; }
        if (!t) {
            fclose(fd);
            err = std::string("Error in file ") + fname + ":   Tag '" + b1 + "' not allowed or multiple defined.";
            return AXS_ERR_PARSE;
        }
        t->seen = true;
        switch (t->type) {
        case FLOAT: *(float *)t->addr = (float)atof(b2); break;
        case INT: *(int *)t->addr = atoi(b2); break;
        case UINT: *(unsigned int *)t->addr = (unsigned int)atoi(b2); break;
        case STRING:
            if (strlen(b2) >= (size_t)kMaxLen) {
                fclose(fd);
                err = std::string("Error in file ") + fname + ": value of tag '" + b1 + "' too long";
                return AXS_ERR_PARSE;
            }
            strcpy((char *)t->addr, b2);
            break;
        }
    }
    fclose(fd);
    for (Tag &x : tags) {
        if (x.required && !x.seen) {
            err = std::string("Error. I miss a value for tag '") + x.name + "' in parameter file '" + fname + "'.";
            return AXS_ERR_PARSE;
        }
    }
    return AXS_OK;
}

axs_params to_params(const RunConfig &c) {
    axs_params p;
    axs_default_params(&p);
    p.lambda = c.lambda;
    p.enable_PRS = c.enable_PRS;
    p.T_initial = c.T_initial;
    p.NDIMS = c.NDIMS;
    p.N = c.N;
    p.space_step = c.space_step;
    p.time_step = c.time_step;
    p.stencil_setting = c.stencil_setting;
    p.seed = c.seed;
    p.thr = c.thr;
    p.precision = c.gpu_precision;
    p.prs = c.gpu_prs;
    p.form = c.gpu_form;
    p.laplacian = c.gpu_laplacian;
    p.tau_initial = 1.0;   // set_physics_variables (src/common/physics.cpp:50)
    return p;
}

}  // namespace axs_host

// Output files in the formats of src/common/fileio.cpp: the main log (stdout
// or a file), snapshot-timings.csv, the time-series CSV, raw field dumps,
// string-position CSVs and power-spectrum CSVs.
#include <cstring>
#include <string>

#include "axs_host.h"

namespace axs_host {

static std::string join(const Output &o, const char *name) { return o.dir + "/" + name; }

int open_outputs(const RunConfig &c, Output &o, std::string &err) {   // fileio.cpp:115-138
    o.dir = c.output_directory;
    if (c.write_output_file) {
        o.main = fopen(c.output_file_path, "w");
        if (!o.main) { err = std::string("cannot open ") + c.output_file_path; return AXS_ERR_ARG; }
    } else {
        o.main = stdout;
    }
    if (c.save_snapshots) {
        std::string p = join(o, "snapshot-timings.csv");
        o.snapshot_timings = fopen(p.c_str(), "w");
        if (!o.snapshot_timings) { err = "cannot open " + p; return AXS_ERR_ARG; }
    }
    if (c.sample_time_series) {
        o.time_series = fopen(c.ts_output_path, "w");
        if (!o.time_series) { err = std::string("cannot open ") + c.ts_output_path; return AXS_ERR_ARG; }
    }
    return AXS_OK;
}

void close_outputs(const RunConfig &c, Output &o) {   // fileio.cpp:140-144
    if (c.write_output_file && o.main && o.main != stdout) fclose(o.main);
    if (o.snapshot_timings) fclose(o.snapshot_timings);
    if (o.time_series) fclose(o.time_series);
    o.snapshot_timings = o.time_series = nullptr;
}

// Raw dump of data_t = double values (the reference's default build).
void save_field_data(Output &o, const char *name, const double *data, long long n) {   // fileio.cpp:15-46
    std::string p = join(o, name);
    fprintf(o.main, "  Saving data... at %s\n", p.c_str());
    FILE *fp = fopen(p.c_str(), "w");
    if (!fp) return;
    fwrite(data, sizeof(double), (size_t)n, fp);
    fclose(fp);
}

void save_strings(Output &o, const char *name, const int *pos, long long n, int ndims) {   // fileio.cpp:83-113
    std::string p = join(o, name);
    fprintf(o.main, "  Saving string positions... at %s\n", p.c_str());
    FILE *fp = fopen(p.c_str(), "w");
    if (!fp) return;
    for (long long q = 0; q < n; ++q) {
        if (ndims == 2) fprintf(fp, "%d, %d\n", pos[2 * q], pos[2 * q + 1]);
        else fprintf(fp, "%d, %d, %d\n", pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]);
    }
    fclose(fp);
}

void save_pk(Output &o, const char *name, const double *pk, const double *ks, const int *count, int nbins) {   // fileio.cpp:64-81
    std::string p = join(o, name);
    fprintf(o.main, "  Saving data... at %s\n", p.c_str());
    FILE *fp = fopen(p.c_str(), "w");
    if (!fp) return;
    fprintf(fp, "k,pk,n_modes\n");
    for (int i = 0; i < nbins; i++)
        if (count[i] != 0) fprintf(fp, "%e,%e,%d\n", ks[i], pk[i], count[i]);
    fclose(fp);
}

void save_axion_spectrum(Output &o, const char *name, const double *k, const double *pk, const long long *count,
                         int nbins) {
    std::string p = join(o, name);
    fprintf(o.main, "  Saving data... at %s\n", p.c_str());
    FILE *fp = fopen(p.c_str(), "w");
    if (!fp) return;
    fprintf(fp, "k,pk,n_modes\n");
    for (int i = 0; i < nbins; i++)
        if (count[i] != 0) fprintf(fp, "%.9e,%.9e,%lld\n", k[i], pk[i], count[i]);
    fclose(fp);
}

}  // namespace axs_host

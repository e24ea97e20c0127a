// axs_run <ParameterFile>: the reference's main + run_standard
// (src/main.cpp:3-26, src/standard/s_run.cpp:26-232) with the lattice on the
// GPU. Same parameter file, same output files and columns; between output
// steps the lattice advances in one axs_evolve call (one CUDA graph replay),
// and only the outputs cross to the host.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "axs_host.h"

namespace axs_host {

namespace {

// physics.cpp:43-74, float results as in the reference
struct Physics {
    float lambda, m_saxion_initial;
    double tau;
    float physical_time() const { return 0.5f * (tau * tau); }
    float scale_factor() const { return (float)tau; }
    float hubble_parameter() const { return 1.0f / (tau * tau); }
    float string_tension() const { return logf(m_saxion_initial / hubble_parameter()); }
};

bool read_file(const char *path, std::vector<unsigned char> &buf) {
    FILE *fp = fopen(path, "rb");
    if (!fp) return false;
    unsigned char chunk[1 << 16];
    size_t n;
    while ((n = fread(chunk, 1, sizeof chunk, fp)) > 0) buf.insert(buf.end(), chunk, chunk + n);
    bool ok = !ferror(fp);
    fclose(fp);
    return ok;
}

bool write_file(const char *path, const std::vector<unsigned char> &buf) {
    FILE *fp = fopen(path, "wb");
    if (!fp) return false;
    bool ok = fwrite(buf.data(), 1, buf.size(), fp) == buf.size();
    return fclose(fp) == 0 && ok;
}

bool every(int tstep, int n, int final_step, int enabled) {   // s_run.cpp:14-24
    if (!enabled) return false;
    int period = final_step / (n - 1);
    return tstep == 0 || (period > 0 && tstep % period == 0);
}

#define CHECK(call)                                                \
    do {                                                           \
        int rc_ = (call);                                          \
        if (rc_ != AXS_OK) {                                       \
            char b_[512];                                          \
            axs_last_error(b_, sizeof b_);                         \
            err = std::string(#call) + ": " + b_;                  \
            return rc_;                                            \
        }                                                          \
    } while (0)

}  // namespace

int run_standard(const RunConfig &c, Output &o, std::string &err) {
    if (c.N % 2 != 0 || (c.NDIMS != 2 && c.NDIMS != 3)) {   // s_run.cpp:32-33
        err = "N must be even and NDIMS 2 or 3";
        return AXS_ERR_ARG;
    }
    axs_params p = to_params(c);
    axs_lattice *h = nullptr;
    CHECK(axs_create(&p, &h));
    struct Guard { axs_lattice *h; ~Guard() { axs_destroy(h); } } guard{h};
    long long length = (c.NDIMS == 3) ? (long long)c.N * c.N * c.N : (long long)c.N * c.N;

    int64_t start_step = 0;
    if (c.gpu_restart_file[0]) {
        // resume: the exact device state of an axs_checkpoint file, at its step
        std::vector<unsigned char> buf;
        if (!read_file(c.gpu_restart_file, buf)) {
            err = std::string("cannot read restart file ") + c.gpu_restart_file;
            return AXS_ERR_ARG;
        }
        CHECK(axs_restore(h, buf.data(), buf.size()));
        CHECK(axs_get_time(h, nullptr, &start_step));
    } else if (c.init_mode == 1) {
        CHECK(axs_init_flat(h, c.seed, c.k_cut));
    } else {
        CHECK(axs_init_gaussian_thermal(h, c.seed));   // s_run.cpp:61
    }

    Physics ph{c.lambda, sqrtf(c.lambda), 1.0};
    if (c.save_snapshots) fprintf(o.snapshot_timings, "snapshot,tau,hubble_scale,string_tension,\n");
    if (c.sample_time_series) {   // s_run.cpp:71-78
        fprintf(o.time_series, "time,scalefactor,");
        if (c.sample_strings) fprintf(o.time_series, "xi,n_plaquettes,");
        if (c.sample_background) fprintf(o.time_series, "phi1_bar,phi2_bar,phidot1_bar,phidot2_bar,axion_bar,saxion_bar");
        fprintf(o.time_series, "\n");
    }

    float lct = 0.5f * c.N * c.space_step;   // physics.cpp:29
    int final_step = (int)(std::round(lct / c.time_step) - std::round(c.space_step / c.time_step) + 1);   // s_run.cpp:82
    if (c.final_step > 0) final_step = c.final_step;

    auto is_output = [&](int t) {
        return every(t, c.n_samples, final_step, c.sample_time_series) ||
               every(t, c.n_snapshots, final_step, c.save_snapshots) ||
               (c.string_interval > 0 && t % c.string_interval == 0) ||
               (c.spectrum_interval > 0 && t % c.spectrum_interval == 0);
    };

    std::vector<double> f1, f2;
    int n_snapshots_written = 0;
    int tstep = (int)start_step;
    while (tstep < final_step) {
        CHECK(axs_get_time(h, &ph.tau, nullptr));
        if (c.check_finite) {
            int fin = 1;
            int rc = axs_check_finite(h, &fin);
            if (!fin || rc == AXS_ERR_NONFINITE) {   // the check of s_run.cpp:4-12
                fprintf(o.main, "Error: NaN encountered in solution vector.\n");
                fprintf(o.main, " tstep = %d\n", tstep);
                err = "NaN encountered";
                return AXS_ERR_NONFINITE;
            }
        }
        if (every(tstep, c.n_samples, final_step, c.sample_time_series)) {   // s_run.cpp:85-153
            fprintf(o.time_series, "%f", ph.physical_time());
            fprintf(o.time_series, ",%f", ph.scale_factor());
            if (c.sample_strings) {
                int64_t nplaq = 0, ncores = 0;
                CHECK(axs_find_strings(h, nullptr, nullptr, &nplaq, &ncores));
                float xi = 0;
                CHECK(axs_xi(&p, nplaq, ncores, ph.tau, &xi));
                fprintf(o.time_series, ",%f", xi);
                fprintf(o.time_series, ",%d", (int)nplaq);
            }
            if (c.sample_background) {
                double m[6];
                CHECK(axs_background(h, m));
                fprintf(o.time_series, ",%f,%f,%f,%f,%f,%f", m[0], m[1], m[2], m[3], m[4], m[5]);
            }
            fprintf(o.time_series, "\n");
        }
        if (every(tstep, c.n_snapshots, final_step, c.save_snapshots)) {   // s_run.cpp:155-211
            fprintf(o.main, "Writing snapshot %d:\n", n_snapshots_written);
            fprintf(o.snapshot_timings, "%d,", n_snapshots_written);
            fprintf(o.snapshot_timings, "%f,", ph.tau);
            fprintf(o.snapshot_timings, "%f,", 1.0f / ph.hubble_parameter());
            fprintf(o.snapshot_timings, "%f,", (c.lambda != 0.0f) ? ph.string_tension() : 0.0f);
            fprintf(o.snapshot_timings, "\n");
            if (c.save_fields) {
                f1.resize(length);
                f2.resize(length);
                CHECK(axs_download(h, f1.data(), f2.data(), nullptr, nullptr));
                char n1[64], n2[64];
                snprintf(n1, sizeof n1, "snapshot%d-phi1", n_snapshots_written);
                snprintf(n2, sizeof n2, "snapshot%d-phi2", n_snapshots_written);
                long long cnt = (c.NDIMS == 2) ? length : (long long)c.N * c.N;   // 3D: first N^2 slice
                save_field_data(o, n1, f1.data(), cnt);
                save_field_data(o, n2, f2.data(), cnt);
            }
            if (c.save_strings) {
                int64_t nplaq = 0, ncores = 0, n = 0;
                CHECK(axs_find_strings(h, nullptr, nullptr, &nplaq, &ncores));
                std::vector<int32_t> pos((size_t)nplaq * c.NDIMS + 1);
                CHECK(axs_string_positions(h, pos.data(), nplaq, &n));
                char nm[64];
                snprintf(nm, sizeof nm, "snapshot%d-strings.csv", n_snapshots_written);
                save_strings(o, nm, pos.data(), n, c.NDIMS);
            }
            if (c.save_pk) {
                int nb = c.N / 2;
                std::vector<double> pk(nb), ks(nb);
                std::vector<int> cnt(nb);
                CHECK(axs_powerspec(h, AXS_PHI2, pk.data(), ks.data(), cnt.data()));
                char nm[64];
                snprintf(nm, sizeof nm, "snapshot%d-pk.csv", n_snapshots_written);
                save_pk(o, nm, pk.data(), ks.data(), cnt.data(), nb);
            }
            n_snapshots_written++;
        }
        if (c.string_interval > 0 && tstep % c.string_interval == 0) {
            int64_t nplaq = 0, ncores = 0;
            CHECK(axs_find_strings(h, nullptr, nullptr, &nplaq, &ncores));
            float xi = 0;
            CHECK(axs_xi(&p, nplaq, ncores, ph.tau, &xi));
            fprintf(o.main, "strings tstep=%d tau=%f n_plaquettes=%lld xi=%f\n", tstep, ph.tau, (long long)nplaq, xi);
        }
        if (c.spectrum_interval > 0 && tstep % c.spectrum_interval == 0) {
            int nb = c.spectrum_bins;
            std::vector<double> k(nb), pk(nb);
            std::vector<long long> cnt(nb);
            CHECK(axs_axion_spectrum(h, nb, k.data(), pk.data(), (int64_t *)cnt.data()));
            char nm[64];
            snprintf(nm, sizeof nm, "axion-spectrum-%06d.csv", tstep);
            save_axion_spectrum(o, nm, k.data(), pk.data(), cnt.data(), nb);
        }
        int next = tstep + 1;
        while (next < final_step && !is_output(next)) ++next;
        CHECK(axs_evolve(h, next - tstep));   // vvsl_field_rescaled x (next - tstep), s_run.cpp:215
        tstep = next;
    }
    if (c.gpu_checkpoint_file[0]) {
        size_t bytes = 0;
        CHECK(axs_checkpoint_size(h, &bytes));
        std::vector<unsigned char> buf(bytes);
        CHECK(axs_checkpoint(h, buf.data(), bytes));
        if (!write_file(c.gpu_checkpoint_file, buf)) {
            err = std::string("cannot write checkpoint file ") + c.gpu_checkpoint_file;
            return AXS_ERR_ARG;
        }
        fprintf(o.main, "  Saving checkpoint... at %s\n", c.gpu_checkpoint_file);
    }
    return AXS_OK;
}

}  // namespace axs_host

int main(int argc, char *argv[]) {
    if (argc != 2) {
        fprintf(stdout, "Error: usage ./axs_run <ParameterFile>\n");
        return EXIT_FAILURE;
    }
    axs_host::RunConfig c;
    std::string err;
    if (axs_host::read_parameter_file(argv[1], c, err) != AXS_OK) {
        printf("%s\n", err.c_str());
        return EXIT_FAILURE;
    }
    if (c.enable_amr) {
        printf("Error: the AMR driver (enable_amr = 1) is not part of the GPU path.\n");
        return EXIT_FAILURE;
    }
    axs_host::Output o;
    if (axs_host::open_outputs(c, o, err) != AXS_OK) {
        printf("%s\n", err.c_str());
        return EXIT_FAILURE;
    }
    fprintf(o.main, "Running with %s\n", argv[1]);
    auto t0 = std::chrono::steady_clock::now();
    int rc = axs_host::run_standard(c, o, err);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (rc != AXS_OK) fprintf(o.main, "Error: %s\n", err.c_str());
    fprintf(o.main, "Time taken: %f seconds\n", secs);
    axs_host::close_outputs(c, o);
    return rc == AXS_OK ? EXIT_SUCCESS : EXIT_FAILURE;
}

/* Thin C entry points over the reference's own hot-path functions, compiled
 * from the reference sources by `make -C oracle ref` (test infrastructure
 * only; the product never loads this library).
 *
 * It stands in for the parts of the reference that the hot path does not
 * contain: it sets the `parameters` global (src/common/common.hpp:30-69)
 * directly instead of parsing a file, and it replaces fio_save_pk
 * (src/common/fileio.cpp:64-81) by a capture of the full-precision arrays so
 * that spectra can be compared beyond the CSV's 7 digits. */
#include <vector>
#include "common/common.hpp"
#include "standard/s_internal.hpp"

FILE *fp_main_output = 0, *fp_time_series = 0, *fp_snapshot_timings = 0;

static std::vector<double> g_pk, g_ks;
static std::vector<int> g_count;

void fio_save_pk(char *file_name, data_t *pk, data_t *ks, int *count, int n_bins) {
    (void)file_name;
    g_pk.assign(pk, pk + n_bins);
    g_ks.assign(ks, ks + n_bins);
    g_count.assign(count, count + n_bins);
}

static all_data g_data;
static bool g_have_matrix = false;
static int g_matrix_dims = 0, g_matrix_n = 0, g_matrix_stencil = -1;

void compute_laplacian_fft(data_t *ret, data_t *field);   // s_integrate.cpp:179 (no header declares it)

extern "C" {

/* compute_laplacian_fft on a caller array (parameters set by ref_set_params). */
void ref_laplacian_fft(data_t *ret, data_t *field) { compute_laplacian_fft(ret, field); }

int ref_sizeof_data_t(void) { return (int)sizeof(data_t); }

void ref_set_params(int ndims, int N, float lambda, float T0, float dx, float dt, int stencil, int thr, unsigned seed) {
    parameters.NDIMS = ndims;
    parameters.N = N;
    parameters.lambda = lambda;
    parameters.enable_PRS = 1;
    parameters.T_initial = T0;
    parameters.space_step = dx;
    parameters.time_step = dt;
    parameters.stencil_setting = stencil;
    parameters.thr = thr;
    parameters.seed = seed;
    set_physics_variables();                           /* physics.cpp:14-35, tau = 1 */
    if (fp_main_output == 0) fp_main_output = stdout;
}

double ref_get_tau(void) { return (double)tau; }
void ref_set_tau(double t) { tau = (data_t)t; }
float ref_meff_squared(void) { return m_eff_squared; }

void ref_gaussian_thermal(data_t *phi1, data_t *phi2, data_t *phidot1, data_t *phidot2) {
    gaussian_thermal(phi1, phi2, phidot1, phidot2);    /* init.cpp:33 */
}

/* n calls of vvsl_field_rescaled (s_integrate.cpp:305), or with form = 1 of
 * vvsl_hamiltonian_form (s_integrate.cpp:358), on caller arrays. */
static void ref_steps_form(data_t *phi1, data_t *phi2, data_t *pd1, data_t *pd2,
                           data_t *k1c, data_t *k2c, data_t *k1n, data_t *k2n, int nsteps, int form) {
    if (!g_have_matrix || g_matrix_dims != parameters.NDIMS || g_matrix_n != parameters.N ||
        g_matrix_stencil != parameters.stencil_setting) {
        if (g_have_matrix) mkl_sparse_destroy(g_data.coefficient_matrix);
        build_coefficient_matrix(&g_data.coefficient_matrix, parameters.NDIMS, parameters.N);
        g_have_matrix = true;
        g_matrix_dims = parameters.NDIMS; g_matrix_n = parameters.N; g_matrix_stencil = parameters.stencil_setting;
    }
    g_data.phi1 = phi1; g_data.phi2 = phi2; g_data.phidot1 = pd1; g_data.phidot2 = pd2;
    g_data.ker1_curr = k1c; g_data.ker2_curr = k2c; g_data.ker1_next = k1n; g_data.ker2_next = k2n;
    g_data.axion = 0; g_data.saxion = 0;
    for (int s = 0; s < nsteps; ++s) {
        if (form == 1) vvsl_hamiltonian_form(g_data);
        else vvsl_field_rescaled(g_data);
    }
}

void ref_steps(data_t *phi1, data_t *phi2, data_t *pd1, data_t *pd2,
               data_t *k1c, data_t *k2c, data_t *k1n, data_t *k2n, int nsteps) {
    ref_steps_form(phi1, phi2, pd1, pd2, k1c, k2c, k1n, k2n, nsteps, 0);
}

void ref_steps_hamiltonian(data_t *phi1, data_t *phi2, data_t *pd1, data_t *pd2,
                           data_t *k1c, data_t *k2c, data_t *k1n, data_t *k2n, int nsteps) {
    ref_steps_form(phi1, phi2, pd1, pd2, k1c, k2c, k1n, k2n, nsteps, 1);
}

/* cores2/cores3 (string_finding.cpp:3-86) on a caller theta array. Writes up
 * to cap positions (2 or 3 ints each) in list order; returns the count. */
int ref_cores(data_t *axion, int *pos, int cap) {
    if (parameters.NDIMS == 2) {
        std::vector<vec2i> s;
        int n = cores2(axion, s);
        for (int q = 0; q < n && q < cap; ++q) { pos[2 * q] = s[q].x; pos[2 * q + 1] = s[q].y; }
        return n;
    }
    std::vector<vec3i> s;
    int n = cores3(axion, s);
    for (int q = 0; q < n && q < cap; ++q) { pos[3 * q] = s[q].x; pos[3 * q + 1] = s[q].y; pos[3 * q + 2] = s[q].z; }
    return n;
}

/* output_powerspec(data_real, NULL) (pk_estimation.cpp:37); N/2 bins. */
void ref_powerspec(data_t *data_real, double *pk, double *ks, int *count) {
    char name[] = "pk.csv";
    output_powerspec(name, data_real, NULL);
    for (size_t b = 0; b < g_pk.size(); ++b) { pk[b] = g_pk[b]; ks[b] = g_ks[b]; count[b] = g_count[b]; }
}

/* xi as printed by run_standard (s_run.cpp:111-114, :123-129). */
float ref_physical_time(void) { return physical_time(); }
float ref_scale_factor(void) { return scale_factor(); }

}

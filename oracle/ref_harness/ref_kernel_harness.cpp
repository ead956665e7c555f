// ref_kernel_harness.cpp -- runs the reference's own kernel-table build on
// the CPU (test infrastructure; used only to pin the oracle and to write
// golden fixtures, never by the engine).
//
// Compiled unmodified from the reference checkout (include path set by
// oracle/ref_harness/build.py):
//   CCCS/DoseCalcIO/spectra.cpp   read_spectrum_file   (spectrum + fluence normalisation)
//   CCCS/DoseCalcIO/kernel.cpp    read_kernel, make_poly_kernel, make_cumulative_kernel
// The HDF5 writer of make_cumulative_kernel lands in the in-memory store of
// oracle/ref_harness/H5Cpp.h; the convolution-angle .raw files it writes go
// to the temp directory given to ccref_kernel_build and are read back with
// the reference's own loaders.  Paths (CCCS/DoseCalcIO/paths.cpp needs
// boost::filesystem) is replaced by the two directories passed in.
#include <cstdlib>
#include <string>

#include "DoseCalcIO/kernel.cpp"
#include "DoseCalcIO/spectra.cpp"

namespace {
std::string g_data_dir, g_temp_dir;
}

Paths* Paths::m_pInstance = nullptr;
Paths* Paths::Instance() {
    if (!m_pInstance) m_pInstance = new Paths;
    m_pInstance->Initialize();
    return m_pInstance;
}
void Paths::Initialize() {
    m_data_dir = g_data_dir;
    m_temp_dir = g_temp_dir;
}

extern "C" {

// One full reference kernel build for `spectrum` (file name without .spec):
// spectrum (normalised fluence), the 48x24 poly kernel (total + 5 categories),
// then the ntheta-bin cumulative kernel with its boundaries and the
// nphi*ntheta/2 convolution angles.  Returns the number of mono kernels, or a
// negative value on a read failure.
int ccref_kernel_build(const char* data_dir, const char* temp_dir, const char* spectrum, int nphi, int ntheta,
                       float* energy, float* fluence, float* mu, float* mu_en, float* poly_total, float* poly_weights,
                       float* cum_total, float* cum_weights, float* radii, float* ang_bounds, float* conv_theta,
                       float* conv_phi) {
    g_data_dir = data_dir;
    g_temp_dir = temp_dir;
    MONO_KERNELS* mono = new MONO_KERNELS;
    KERNEL* poly = new KERNEL;
    mono->spectrum_file = spectrum;
    int rc = -1;
    if (read_spectrum_file(mono, false) != 1) goto done;
    for (int i = 0; i < mono->nkernels; i++)
        if (read_kernel(&mono->kernel[i]) != 1) goto done;
    if (make_poly_kernel(mono, poly, 0, 0) != 1) goto done;
    for (int i = 0; i < mono->nkernels; i++) {
        energy[i] = mono->energy[i];
        fluence[i] = mono->fluence[i];
        mu[i] = mono->mu[i];
        mu_en[i] = mono->mu_en[i];
    }
    {
        const int n = poly->ntheta * poly->nradii;
        std::memcpy(poly_total, poly->total_matrix.data(), n * sizeof(float));
        for (int c = 0; c < N_KERNEL_CATEGORIES; c++)
            std::memcpy(poly_weights + c * n, poly->matrix[c].data(), n * sizeof(float));
    }
    H5::mem_datasets.clear();
    H5::mem_attrs.clear();
    if (make_cumulative_kernel(poly, nphi, ntheta, 0) != 1) goto done;
    {
        const H5::MemArray& t = H5::mem_datasets["total_weights"];
        const H5::MemArray& w = H5::mem_datasets["weights"];
        std::memcpy(cum_total, t.bytes.data(), t.bytes.size());
        std::memcpy(cum_weights, w.bytes.data(), w.bytes.size());
        const H5::MemArray& r = H5::mem_attrs["radial_boundaries_cm"];
        const H5::MemArray& a = H5::mem_attrs["angular_boundaries_deg"];
        std::memcpy(radii, r.bytes.data(), r.bytes.size());
        std::memcpy(ang_bounds, a.bytes.data(), a.bytes.size());
        const int numangles = nphi * ntheta / 2;
        float *th = nullptr, *ph = nullptr;
        if (!load_convolution_theta_angles(&th, numangles) || !load_convolution_phi_angles(&ph, numangles)) goto done;
        std::memcpy(conv_theta, th, numangles * sizeof(float));
        std::memcpy(conv_phi, ph, numangles * sizeof(float));
        delete[] th;
        delete[] ph;
    }
    rc = mono->nkernels;
done:
    delete poly;
    delete mono;
    return rc;
}

}  // extern "C"

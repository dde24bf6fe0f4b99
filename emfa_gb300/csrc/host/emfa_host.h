// C++ host front end with the reference's class surface (xiangwei0909/EMFA):
// ConfigLoader (EMComponent/ConfigLoader.h), Mesh NAS input
// (EMComponent/Mesh.cpp:261-309,727-779), Result RCS writers
// (EMComponent/Result.h:47-155), the EM solver lifecycle
// init / reportInfo / solve / output / clear (EMSolver/EM.h:21-54,
// EMSolver/Solver.h:20-29) for EFIE, CFIE and MLFMA, and
// solver::loadSolver (EMSolver/Solver.cpp:45-95).  Every numerical stage
// runs through the C ABI of libemfa_cuda.so (include/emfa_cuda.h).
#pragma once

#include <chrono>
#include <complex>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../../include/emfa_cuda.h"

namespace component {

// EMComponent/ErrorHandle.h:11-21
class ConfigInvalid : public std::invalid_argument {
public:
    explicit ConfigInvalid(const std::string& s) : std::invalid_argument(s) {}
};
class FileError : public std::runtime_error {
public:
    explicit FileError(const std::string& s) : std::runtime_error(s) {}
};

namespace policy {
enum ResultType { BiRCS = 0, MonoRCS, Rad };
}

struct Incidence {
    float freq, freq_from, freq_to, freq_delta, freq_inc, theta, phi, pole;
};
struct Scattering {
    float theta_from, theta_to, theta_delta, phi_from, phi_to, phi_delta;
};

// `key: value` token file with '#' comment lines (ConfigLoader.cpp:23-50).
// Values parse lazily with std::stof / std::stoi as the reference does; a
// missing key throws std::out_of_range from the dictionary lookup.
class ConfigLoader {
public:
    void load(const std::string& path);
    std::string getSolverType();
    Incidence getInc();
    policy::ResultType getResultType();
    Scattering getSca();
    void getNearfield();  // read (and validated) by EM::init in the reference
    std::string getMeshPath();
    float getAlpha();
    float getIterationThreshold();
    int getMaxIterationNum();
    float getMLFMABoxThreshold();
    bool getPreconditioningSwitch();
    float getRowThreshold();
    float getColThreshold();
    size_t getThreadNumber();
    size_t getTaskFactor();
    std::complex<float> getSigma();
    float getDx();
    float getDy();
    int getArray_x();
    int getArray_y();
    // build-only keys (prefix gpu_, ignored by the reference)
    std::string getGpu(const std::string& key, const std::string& dflt) const;
    const std::string& getReport() const { return report_; }
    bool has(const std::string& k) const { return dict_.count(k) != 0; }

private:
    const std::string& at(const std::string& k);
    float f(const std::string& k, const char* what);
    std::map<std::string, std::string> dict_;
    std::string report_;
};

// Mesh read from the NAS subset the reference parses; coordinates pass
// through the same 6-significant-digit text round trip.
struct Mesh {
    std::vector<double> verts;  // V x 3
    std::vector<int> tris;      // T x 3, 0-based
    void loadMeshFile(const std::string& path);
    int nodes() const { return (int)verts.size() / 3; }
    int triangles() const { return (int)tris.size() / 3; }
};

}  // namespace component

namespace mom {

class EM {
public:
    virtual ~EM();
    virtual void init(component::ConfigLoader* ploader);
    virtual void solve() {}
    virtual void output() {}
    virtual void clear();
    virtual void reportInfo(std::ostream& strm) const;
    const std::string& outputDir() const { return dir_; }

protected:
    void timeLog(const std::string& what);
    void openContext(component::ConfigLoader* ploader);
    void writeBistatic(const emfa_fill_params_t& fp, const void* I_dev);
    // MonostaticRCS: one incidence per direction of Result::getMonostaticRCS
    // (EMComponent/Result.h:106-155), in its order -- the phi cuts over theta,
    // then the theta = 90 ring -- each seen from its backscatter direction
    void planMonostatic();
    void writeMonostatic(const emfa_fill_params_t& fp, const void* I_dev);
    // the run's incidences (theta, phi, pole in degrees, n_inc_ of them)
    std::vector<double> inc_angles_;
    int n_inc_ = 1;
    struct RcsFile {
        std::string name;
        std::vector<float> angles;
    };
    std::vector<RcsFile> mono_files_;
    std::vector<double> mono_dirs_;  // n_inc_ x 3, the backscatter direction of each incidence
    component::policy::ResultType rtype_ = component::policy::BiRCS;
    component::Incidence incidence_{};
    component::Scattering scattering_{};
    std::string dir_, folder_name_;
    std::ofstream logger_;
    std::ostringstream time_log_;
    std::chrono::steady_clock::time_point t_start_, t_prev_;
    component::Mesh mesh_;
    std::vector<int> rwg_;
    int unknowns_ = 0;
    emfa_ctx_t* ctx_ = nullptr;
    emfa_geom_t* geom_ = nullptr;
    int precision_ = EMFA_F32;
};

class EFIE : public EM {
public:
    void init(component::ConfigLoader* ploader) override;
    void solve() override;
    void output() override;
    void clear() override;

private:
    std::complex<float> sigma_;
    float tol_ = 1e-3f;
    int disc_ = EMFA_DISC_REFERENCE;  // gpu_discretisation: reference | config
    void* Z_ = nullptr;
    void* V_ = nullptr;
    void* I_ = nullptr;
};

class CFIE : public EM {
public:
    void init(component::ConfigLoader* ploader) override;
    void solve() override;
    void output() override;
    void clear() override;

private:
    float alpha_ = 1.0f;
    float tol_ = 0.01f;
    void* Z_ = nullptr;
    void* V_ = nullptr;
    void* I_ = nullptr;
    int iterations_ = 0;
};

// MLFMA (EMSolver/MLFMA.cpp:23-131): CFIE operator with the multilevel fast
// multipole far field, BiCGStab to iteration_threshold (box order).
class MLFMA : public EM {
public:
    ~MLFMA() override
    {
        if (ml_) emfa_mlfma_destroy(ml_);
    }
    void init(component::ConfigLoader* ploader) override;
    void solve() override;
    void output() override;
    void clear() override;
    void reportInfo(std::ostream& strm) const override;

private:
    float alpha_ = 1.0f, threshold_ = 0.25f, tol_ = 1e-3f;
    int max_iter_ = 500;
    bool precond_ = false;
    emfa_mlfma_t* ml_ = nullptr;
    void* V_ = nullptr;
    void* Ibox_ = nullptr;
    void* I_ = nullptr;
    int levels_ = 0;
};

}  // namespace mom

namespace solver {
// EMSolver/Solver.cpp:45-95: dispatch on `EMSolver:` and run
// init -> reportInfo -> solve -> output -> clear (Solver.h:20-29)
void loadSolver(const std::string& conf_file);
}  // namespace solver

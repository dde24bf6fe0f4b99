// C++ host front end: the reference's solver surface over libemfa_cuda.so.
#include "emfa_host.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <iomanip>
#include <iostream>
#include <limits>

namespace component {

// ---------------------------------------------------------------------------
// ConfigLoader (EMComponent/ConfigLoader.cpp)
// ---------------------------------------------------------------------------
void ConfigLoader::load(const std::string& path)
{
    std::ifstream config(path);
    if (config.fail()) throw ConfigInvalid("fail opening config file(" + path + ')');
    const auto max_len = std::numeric_limits<std::streamsize>::max();
    auto skip = [&]() {
        for (auto ch = config.peek(); std::isspace(ch) || ch == '#'; ch = config.peek()) {
            if (ch == '#')
                config.ignore(max_len, '\n');
            else
                config.get();
        }
    };
    skip();
    std::string key, value;
    while (config >> key >> value) {
        dict_[key] = value;
        skip();
    }
}

const std::string& ConfigLoader::at(const std::string& k)
{
    auto it = dict_.find(k);
    if (it == dict_.end()) throw std::out_of_range("map::at (config key " + k + ")");
    report_ += "    " + k + " " + it->second + "\n";
    return it->second;
}

float ConfigLoader::f(const std::string& k, const char* what)
{
    const std::string& v = at(k);
    try {
        return std::stof(v);
    } catch (...) {
        throw ConfigInvalid(what);
    }
}

std::string ConfigLoader::getSolverType() { return at("EMSolver:"); }

Incidence ConfigLoader::getInc()
{
    Incidence inc;
    const char* w = "fail parsing incidence information";
    inc.freq = f("frequency:", w);
    inc.freq_from = f("frequency_from:", w);
    inc.freq_to = f("frequency_to:", w);
    inc.freq_delta = f("frequency_delta:", w);
    inc.freq_inc = f("frequency_inc:", w);
    inc.theta = f("theta:", w);
    inc.phi = f("phi:", w);
    inc.pole = f("pole:", w);
    return inc;
}

policy::ResultType ConfigLoader::getResultType()
{
    const std::string& v = at("result_type:");
    if (v == "BistaticRCS") return policy::BiRCS;
    if (v == "MonostaticRCS") return policy::MonoRCS;
    if (v == "Radiation") return policy::Rad;
    throw ConfigInvalid("type parameter only supports three type values (BistaticRCS, MonostaticRCS and Radiation)");
}

Scattering ConfigLoader::getSca()
{
    Scattering s;
    const char* w = "fail parsing scattering information";
    s.theta_from = f("theta_from:", w);
    s.theta_to = f("theta_to:", w);
    s.theta_delta = f("theta_delta:", w);
    s.phi_from = f("phi_from:", w);
    s.phi_to = f("phi_to:", w);
    s.phi_delta = f("phi_delta:", w);
    return s;
}

void ConfigLoader::getNearfield()
{
    for (const char* k : {"Origin_point:", "End_point:"}) {
        const std::string& v = at(k);
        auto p1 = v.find_first_of('('), p2 = v.find_first_of(','), p3 = v.find_last_of(','), p4 = v.find_last_of(')');
        try {
            std::stof(v.substr(p1 + 1, p2 - p1 - 1));
            std::stof(v.substr(p2 + 1, p3 - p2 - 1));
            std::stof(v.substr(p3 + 1, p4 - p3 - 1));
        } catch (...) {
            throw ConfigInvalid(std::string("fail parsing ") + (k[0] == 'O' ? "Origin point" : "end point"));
        }
    }
    for (const char* k : {"Sampling_x:", "Sampling_y:", "Sampling_z:"}) {
        try {
            std::stoi(at(k));
        } catch (const std::out_of_range&) {
            throw;
        } catch (...) {
            throw ConfigInvalid("fail parsing sampling number");
        }
    }
}

std::string ConfigLoader::getMeshPath() { return at("mesh_path:"); }
float ConfigLoader::getAlpha() { return f("alpha:", "fail parsing combined coefficient"); }
float ConfigLoader::getIterationThreshold() { return f("iteration_threshold:", "fail parsing iteration threshold"); }
int ConfigLoader::getMaxIterationNum()
{
    try {
        return std::stoi(at("max_iteration_number:"));
    } catch (const std::out_of_range&) {
        throw;
    } catch (...) {
        throw ConfigInvalid("fail parsing maximum iteration number");
    }
}
float ConfigLoader::getMLFMABoxThreshold() { return f("mlfma_box_threshold:", "fail parsing MLFMA box threshold"); }
bool ConfigLoader::getPreconditioningSwitch()
{
    const std::string& v = at("preconditioning:");
    if (v == "true") return true;
    if (v == "false") return false;
    throw ConfigInvalid("Precondition switch only supports two options (true or false)");
}
float ConfigLoader::getRowThreshold()
{
    float v = f("row_threshold:", "fail parsing row threshold");
    if (v < 0.87f) throw ConfigInvalid("row threshold parameter cannot less than 0.87");
    return v;
}
float ConfigLoader::getColThreshold()
{
    float v = f("col_threshold:", "fail parsing column threshold");
    if (v < 0.87f) throw ConfigInvalid("column threshold parameter cannot less than 0.87");
    return v;
}
size_t ConfigLoader::getThreadNumber()
{
    try {
        return std::stoull(at("thread_number:"));
    } catch (const std::out_of_range&) {
        throw;
    } catch (...) {
        throw ConfigInvalid("fail parsing thread number");
    }
}
size_t ConfigLoader::getTaskFactor()
{
    try {
        return std::stoull(at("task_factor:"));
    } catch (const std::out_of_range&) {
        throw;
    } catch (...) {
        throw ConfigInvalid("fail parsing task factor");
    }
}
std::complex<float> ConfigLoader::getSigma()
{
    const std::string& v = at("Sigma:");
    auto p1 = v.find_first_of('('), p2 = v.find_first_of(','), p3 = v.find_first_of(')');
    try {
        return {std::stof(v.substr(p1 + 1, p2 - p1 - 1)), std::stof(v.substr(p2 + 1, p3 - p2 - 1))};
    } catch (...) {
        throw ConfigInvalid("fail parsing sigma");
    }
}
float ConfigLoader::getDx() { return f("Dx:", "fail parsing Dx"); }
float ConfigLoader::getDy() { return f("Dy:", "fail parsing Dy"); }
int ConfigLoader::getArray_x()
{
    try {
        return std::stoi(at("Array_x:"));
    } catch (const std::out_of_range&) {
        throw;
    } catch (...) {
        throw ConfigInvalid("fail parsing Array_x");
    }
}
int ConfigLoader::getArray_y()
{
    try {
        return std::stoi(at("Array_y:"));
    } catch (const std::out_of_range&) {
        throw;
    } catch (...) {
        throw ConfigInvalid("fail parsing Array_y");
    }
}
std::string ConfigLoader::getGpu(const std::string& key, const std::string& dflt) const
{
    auto it = dict_.find(key);
    return it == dict_.end() ? dflt : it->second;
}

// ---------------------------------------------------------------------------
// Mesh: Mesh::loadNasFile / readNasTmpFile (EMComponent/Mesh.cpp:261-309,
// 727-779).  Nine header lines, GRID* + '*' continuation, CTRIA3, ENDDATA;
// ids must run 1, 2, 3, ...; each coordinate is read as float and
// re-read from its default-precision (6 significant digits) text form.
// ---------------------------------------------------------------------------
static double six_digits(double v)
{
    std::ostringstream o;
    o << v;  // default stream precision, as the reference's temp file
    return std::stod(o.str());
}

void Mesh::loadMeshFile(const std::string& path)
{
    std::string suffix = path.substr(path.find_last_of('.') + 1);
    if (suffix != "nas")
        throw FileError("cannot identify mesh file type: " + suffix + " (only .nas meshes are read)");
    std::ifstream in(path);
    if (in.fail()) throw FileError("fail loading nas mesh file: " + path);
    const auto maxs = std::numeric_limits<std::streamsize>::max();
    for (int t = 0; t < 9; ++t) in.ignore(maxs, '\n');
    int node_num = 0, tri_num = 0;
    while (in.peek() != 'E') {
        if (in.peek() == std::char_traits<char>::eof()) throw FileError("fail loading nas mesh file: " + path);
        bool any = false;
        while (in.peek() == 'G') {
            int id;
            double x, y, z;
            in.ignore(maxs, '*');
            in >> id >> x >> y;
            in.ignore(maxs, '*');
            in >> id >> z;
            if (!in || id != ++node_num) throw FileError("fail loading nas mesh file: " + path);
            verts.insert(verts.end(), {six_digits(x), six_digits(y), six_digits(z)});
            in.get();
            any = true;
        }
        while (in.peek() == 'C') {
            int id, group, a, b, c;
            in.ignore(maxs, ' ');
            in >> id >> group >> a >> b >> c;
            if (!in || id != ++tri_num) throw FileError("fail loading nas mesh file: " + path);
            tris.insert(tris.end(), {a - 1, b - 1, c - 1});
            in.get();
            any = true;
        }
        if (!any) throw FileError("fail loading nas mesh file: " + path);
    }
    for (int v : tris)
        if (v < 0 || v >= node_num) throw FileError("fail reading nas temp file");
}

}  // namespace component

// ---------------------------------------------------------------------------
// solvers
// ---------------------------------------------------------------------------
namespace mom {

using namespace component;

static void check(emfa_status_t s, emfa_ctx_t* ctx, const char* what)
{
    if (s == EMFA_OK) return;
    std::string msg = std::string(what) + ": " + emfa_status_string(s) + " (" + emfa_last_error(ctx) + ")";
    if (s == EMFA_ERR_INVALID) throw ConfigInvalid(msg);
    if (s == EMFA_ERR_MESH) throw FileError(msg);
    throw std::runtime_error(msg);
}

EM::~EM()
{
    if (geom_) emfa_geom_destroy(geom_);
    if (ctx_) emfa_ctx_destroy(ctx_);
}

void EM::timeLog(const std::string& what)
{
    auto now = std::chrono::steady_clock::now();
    long long ms = std::chrono::duration_cast<std::chrono::milliseconds>(now - t_prev_).count();
    t_prev_ = now;
    std::ostringstream o;
    o << std::left << std::setw(30) << ("Time of " + what + ":") << std::right << std::setw(12) << ms << " ms\n";
    time_log_ << o.str();
    if (logger_.is_open()) logger_ << o.str() << std::flush;
    std::cout << o.str() << std::flush;
}

// EM::init (EMSolver/EM.cpp:24-67)
void EM::init(ConfigLoader* ploader)
{
    t_start_ = t_prev_ = std::chrono::steady_clock::now();
    rtype_ = ploader->getResultType();
    incidence_ = ploader->getInc();
    if (rtype_ == policy::Rad) throw ConfigInvalid("only scattering results (BistaticRCS) are computed");
    scattering_ = ploader->getSca();
    ploader->getNearfield();
    std::string mesh_file = ploader->getMeshPath();
    auto pos_suffix = mesh_file.find_last_of('.');
    if (pos_suffix == std::string::npos) throw ConfigInvalid("mesh path parameter cannot match");
    auto p1 = mesh_file.find_last_of('/'), p2 = mesh_file.find_last_of('\\');
    if (p1 == std::string::npos && p2 == std::string::npos) {
        dir_ = ".";
        folder_name_ = mesh_file.substr(0, pos_suffix);
    } else {
        auto pd = (p1 != std::string::npos && p2 != std::string::npos) ? std::max(p1, p2) : std::min(p1, p2);
        dir_ = mesh_file.substr(0, pd);
        folder_name_ = mesh_file.substr(pd + 1, pos_suffix - pd - 1);
    }
    inc_angles_ = {incidence_.theta, incidence_.phi, incidence_.pole};
    n_inc_ = 1;
    if (rtype_ == policy::MonoRCS) planMonostatic();
    mesh_.loadMeshFile(mesh_file);
    int cap = 3 * mesh_.triangles() / 2 + 16, n = 0;
    rwg_.assign((size_t)6 * cap, 0);
    check(emfa_build_rwg(mesh_.tris.data(), mesh_.triangles(), rwg_.data(), cap, &n), nullptr, "CommonEdge");
    rwg_.resize((size_t)6 * n);
    unknowns_ = n;
    openContext(ploader);
}

void EM::openContext(ConfigLoader* ploader)
{
    int device = std::atoi(ploader->getGpu("gpu_device:", "0").c_str());
    size_t budget = (size_t)std::atof(ploader->getGpu("gpu_hbm_budget_gb:", "0").c_str()) * (1ull << 30);
    precision_ = ploader->getGpu("gpu_precision:", "f32") == "f64" ? EMFA_F64 : EMFA_F32;
    check(emfa_ctx_create(device, budget, &ctx_), nullptr, "emfa_ctx_create");
    check(emfa_geom_create(ctx_, mesh_.verts.data(), mesh_.nodes(), mesh_.tris.data(), mesh_.triangles(),
                           rwg_.data(), unknowns_, &geom_),
          ctx_, "emfa_geom_create");
}

void EM::clear()
{
    if (geom_) emfa_geom_destroy(geom_);
    geom_ = nullptr;
    rwg_.clear();
    mesh_ = Mesh();
}

void EM::reportInfo(std::ostream& strm) const
{
    strm << "Mesh Information\n    Vertices: " << mesh_.nodes() << "\n    Triangles: " << mesh_.triangles()
         << "\nCommonEdge Information\n    Total RWGs: " << unknowns_ << '\n';
}

// Result::getBistaticRCS (EMComponent/Result.h:47-104): one file per phi cut
// over theta, plus the theta = 90 ring.  All directions go to the device in
// one emfa_rcs call; the files keep the reference's layout and precision.
void EM::writeBistatic(const emfa_fill_params_t& fp, const void* I_dev)
{
    const float d2r = 3.14159265358979323846f / 180.0f;
    std::vector<double> dirs;
    std::vector<std::pair<std::string, std::vector<float>>> files;
    const auto& sca = scattering_;
    int num = static_cast<int>((sca.phi_to - sca.phi_from) / sca.phi_delta + 1);
    for (int i = 0; i < num; ++i) {
        float phi_deg = sca.phi_from + i * sca.phi_delta;
        float phi = phi_deg * d2r;
        float cosp = (float)std::cos((double)phi), sinp = (float)std::sin((double)phi);
        std::string str = std::to_string(phi_deg);
        files.push_back({"bistatic_rcs_phi_" + str.substr(0, str.find('.')) + ".dat", {}});
        for (float td = sca.theta_from; td <= sca.theta_to; td += sca.theta_delta) {
            double th = (double)(td * d2r);
            dirs.insert(dirs.end(), {(double)(float)(std::sin(th) * cosp), (double)(float)(std::sin(th) * sinp),
                                     (double)(float)std::cos(th)});
            files.back().second.push_back(td);
        }
    }
    files.push_back({"bistatic_rcs_theta_90.dat", {}});
    for (float pd = 0; pd < 360; pd += 1) {
        double p = (double)(pd * d2r);
        dirs.insert(dirs.end(), {(double)(float)std::cos(p), (double)(float)std::sin(p), 0.0});
        files.back().second.push_back(pd);
    }
    int nd = (int)dirs.size() / 3;
    std::vector<double> rcs(nd);
    check(emfa_rcs(ctx_, geom_, &fp, I_dev, 1, dirs.data(), nd, 0, rcs.data(), nullptr), ctx_, "emfa_rcs");
    size_t k = 0;
    for (auto& fl : files) {
        std::ofstream o(dir_ + "/" + fl.first);
        o << std::right << std::fixed << std::setprecision(4);
        o << std::setw(10) << "Theta\t" << std::setw(10) << "RCS(dBm^2)\n";
        for (float ang : fl.second) o << std::setw(10) << ang << '\t' << std::setw(10) << (float)rcs[k++] << '\n';
    }
}

// The sweep of Result::getMonostaticRCS (EMComponent/Result.h:106-155): for
// each phi cut the theta rows, then phi = 0..359 at theta = 90, in float
// arithmetic as the reference steps its angles.  Direction (theta, phi) is
// seen from the incidence at the same angles: the reference's incident wave
// travels along -r_hat(theta, phi) (EMSolver/EM.cpp:33), so the backscatter
// direction is r_hat(theta, phi); the polarisation is the config's pole.
void EM::planMonostatic()
{
    const float d2r = 3.14159265358979323846f / 180.0f;
    const auto& sca = scattering_;
    inc_angles_.clear();
    mono_dirs_.clear();
    mono_files_.clear();
    int phi_num = static_cast<int>((sca.phi_to - sca.phi_from) / sca.phi_delta) + 1;
    for (int i = 0; i < phi_num; ++i) {
        float phi_deg = sca.phi_from + i * sca.phi_delta;
        float phi = phi_deg * d2r;
        float cosp = (float)std::cos((double)phi), sinp = (float)std::sin((double)phi);
        std::string str = std::to_string(phi_deg);
        mono_files_.push_back({"monostatic_rcs_phi_" + str.substr(0, str.find('.')) + ".dat", {}});
        for (float td = sca.theta_from; td <= sca.theta_to; td += sca.theta_delta) {
            double th = (double)(td * d2r);
            mono_dirs_.insert(mono_dirs_.end(), {(double)(float)(std::sin(th) * cosp),
                                                 (double)(float)(std::sin(th) * sinp), (double)(float)std::cos(th)});
            inc_angles_.insert(inc_angles_.end(), {(double)td, (double)phi_deg, (double)incidence_.pole});
            mono_files_.back().angles.push_back(td);
        }
    }
    mono_files_.push_back({"monostatic_rcs_theta_90.dat", {}});
    for (float pd = 0; pd < 360; pd += 1) {
        double p = (double)(pd * d2r);
        mono_dirs_.insert(mono_dirs_.end(), {(double)(float)std::cos(p), (double)(float)std::sin(p), 0.0});
        inc_angles_.insert(inc_angles_.end(), {90.0, (double)pd, (double)incidence_.pole});
        mono_files_.back().angles.push_back(pd);
    }
    n_inc_ = (int)inc_angles_.size() / 3;
    if (n_inc_ > 65535) throw ConfigInvalid("monostatic sweep: more than 65535 incidences");
}

// One emfa_rcs call for all incidences, each at its own backscatter
// direction; the files keep the reference's layout (same header and columns
// as the bistatic files).
void EM::writeMonostatic(const emfa_fill_params_t& fp, const void* I_dev)
{
    std::vector<double> rcs(n_inc_);
    check(emfa_rcs(ctx_, geom_, &fp, I_dev, n_inc_, mono_dirs_.data(), 1, 1, rcs.data(), nullptr), ctx_,
          "emfa_rcs");
    size_t k = 0;
    for (auto& fl : mono_files_) {
        std::ofstream o(dir_ + "/" + fl.name);
        o << std::right << std::fixed << std::setprecision(4);
        o << std::setw(10) << "Theta\t" << std::setw(10) << "RCS(dBm^2)\n";
        for (float ang : fl.angles) o << std::setw(10) << ang << '\t' << std::setw(10) << (float)rcs[k++] << '\n';
    }
}

static std::string make_folder(const std::string& dir, const std::string& name)
{
    std::string d = dir + '/' + name;
    std::filesystem::create_directory(d);
    return d;
}

// EFIE (EMSolver/EFIE.cpp:25-119): GMRES(30) to an absolute 1e-3
void EFIE::init(ConfigLoader* ploader)
{
    EM::init(ploader);
    dir_ = make_folder(dir_, folder_name_ + "_EFIE");
    logger_.open(dir_ + "/sca_runtime.log");
    sigma_ = ploader->getSigma();
    ploader->getDx();
    ploader->getDy();
    ploader->getArray_x();
    ploader->getArray_y();
    tol_ = std::atof(ploader->getGpu("gpu_efie_tol:", "1e-3").c_str());
    const std::string disc = ploader->getGpu("gpu_discretisation:", "reference");
    if (disc != "reference" && disc != "config")
        throw ConfigInvalid("gpu_discretisation: must be reference or config");
    disc_ = disc == "config" ? EMFA_DISC_CONFIG : EMFA_DISC_REFERENCE;
    logger_ << ploader->getReport();
    reportInfo(logger_);
    timeLog("init");
}

void EFIE::solve()
{
    const size_t es = precision_ == EMFA_F64 ? 16 : 8;
    const size_t n = unknowns_, r = n_inc_;
    check(emfa_device_alloc(ctx_, es * n * n, &Z_), ctx_, "alloc Z");
    check(emfa_device_alloc(ctx_, es * n * r, &V_), ctx_, "alloc V");
    check(emfa_device_alloc(ctx_, 16 * n * r, &I_), ctx_, "alloc I");
    emfa_fill_params_t fp{EMFA_EFIE, precision_, (double)incidence_.freq, 1.0, sigma_.real(), sigma_.imag(), 0, disc_};
    check(emfa_fill_z(ctx_, geom_, &fp, Z_, n, nullptr), ctx_, "fillZ");
    timeLog("fillZ");
    check(emfa_fill_v(ctx_, geom_, &fp, inc_angles_.data(), n_inc_, V_, nullptr), ctx_, "fillV");
    timeLog("fillV");
    emfa_solver_params_t sp{EMFA_GMRES, 30, 100000, tol_, 1, EMFA_MV_AUTO, 0, 0};
    emfa_solve_info_t info{};
    emfa_status_t s = emfa_solve(ctx_, precision_, Z_, (int)n, V_, n_inc_, I_, &sp, &info, nullptr);
    if (s == EMFA_ERR_NOT_CONVERGED)
        logger_ << "    WARNING: Iteration cannot converge\n";
    else
        check(s, ctx_, "GMRES");
    logger_ << "    Iterative number: " << info.iterations << '\n';
    std::cout << "  -> Iterative number: " << info.iterations << std::endl;
    timeLog("solve");
}

void EFIE::output()
{
    emfa_fill_params_t fp{EMFA_EFIE, precision_, (double)incidence_.freq, 1.0, sigma_.real(), sigma_.imag(), 0, disc_};
    if (rtype_ == policy::MonoRCS) {
        writeMonostatic(fp, I_);
        timeLog("getMonostaticRCS");
    } else {
        writeBistatic(fp, I_);
        timeLog("getBistaticRCS");
    }
}

void EFIE::clear()
{
    for (void* p : {Z_, V_, I_})
        if (p) emfa_device_free(ctx_, p);
    Z_ = V_ = I_ = nullptr;
    EM::clear();
}

// CFIE (EMSolver/CFIE.cpp:25-110): BiCGStab to 1e-2 relative, 500 iterations
void CFIE::init(ConfigLoader* ploader)
{
    EM::init(ploader);
    alpha_ = ploader->getAlpha();
    tol_ = std::atof(ploader->getGpu("gpu_cfie_tol:", "0.01").c_str());
    dir_ = make_folder(dir_, folder_name_ + "_CFIE_" + std::to_string(alpha_).substr(0, 3));
    logger_.open(dir_ + "/sca_runtime.log");
    logger_ << ploader->getReport();
    reportInfo(logger_);
    timeLog("init");
}

void CFIE::solve()
{
    const size_t es = precision_ == EMFA_F64 ? 16 : 8;
    const size_t n = unknowns_, r = n_inc_;
    check(emfa_device_alloc(ctx_, es * n * n, &Z_), ctx_, "alloc Z");
    check(emfa_device_alloc(ctx_, es * n * r, &V_), ctx_, "alloc V");
    check(emfa_device_alloc(ctx_, 16 * n * r, &I_), ctx_, "alloc I");
    emfa_fill_params_t fp{EMFA_CFIE, precision_, (double)incidence_.freq, (double)alpha_, 0, 0, 0};
    check(emfa_fill_z(ctx_, geom_, &fp, Z_, n, nullptr), ctx_, "fillZ");
    timeLog("fillZ");
    check(emfa_fill_v(ctx_, geom_, &fp, inc_angles_.data(), n_inc_, V_, nullptr), ctx_, "fillV");
    timeLog("fillV");
    emfa_solver_params_t sp{EMFA_BICGSTAB, 30, 500, tol_, 0, EMFA_MV_AUTO, 0, 0};
    emfa_solve_info_t info{};
    emfa_status_t s = emfa_solve(ctx_, precision_, Z_, (int)n, V_, n_inc_, I_, &sp, &info, nullptr);
    if (s == EMFA_ERR_NOT_CONVERGED)
        logger_ << "    WARNING: Iteration cannot converge\n";
    else
        check(s, ctx_, "BiCGStab");
    iterations_ = info.iterations;
    logger_ << "    Iterative number: " << iterations_ << '\n';
    std::cout << "    Iterative number: " << iterations_ << std::endl;
    timeLog("solve");
}

void CFIE::output()
{
    emfa_fill_params_t fp{EMFA_CFIE, precision_, (double)incidence_.freq, (double)alpha_, 0, 0, 0};
    if (rtype_ == policy::MonoRCS) {
        writeMonostatic(fp, I_);
        timeLog("getMonostaticRCS");
    } else {
        writeBistatic(fp, I_);
        timeLog("getBistaticRCS");
    }
}

void CFIE::clear()
{
    for (void* p : {Z_, V_, I_})
        if (p) emfa_device_free(ctx_, p);
    Z_ = V_ = I_ = nullptr;
    EM::clear();
}

void MLFMA::init(ConfigLoader* ploader)
{
    EM::init(ploader);
    alpha_ = ploader->getAlpha();
    dir_ = make_folder(dir_, folder_name_ + "_MLFMA_CFIE_" + std::to_string(alpha_).substr(0, 3));
    logger_.open(dir_ + "/sca_parallel_runtime.log");
    tol_ = ploader->getIterationThreshold();
    max_iter_ = ploader->getMaxIterationNum();
    precond_ = ploader->getPreconditioningSwitch();
    const float row_thr = ploader->getRowThreshold();
    const float col_thr = ploader->getColThreshold();
    threshold_ = ploader->getMLFMABoxThreshold();
    ploader->getThreadNumber();
    ploader->getTaskFactor();
    const std::string trunc = ploader->getGpu("gpu_mlfma_truncation:", "reference");
    if (trunc != "reference" && trunc != "config")
        throw ConfigInvalid("gpu_mlfma_truncation: must be reference or config");
    emfa_mlfma_params_t mp{(double)incidence_.freq, (double)alpha_, (double)threshold_, precond_ ? 1 : 0,
                           (double)row_thr, (double)col_thr, trunc == "config" ? 1 : 0};
    check(emfa_mlfma_create(ctx_, geom_, &mp, &ml_), ctx_, "MLFMA init");
    check(emfa_mlfma_info(ml_, &levels_, nullptr, nullptr, nullptr, nullptr), ctx_, "MLFMA info");
    logger_ << ploader->getReport();
    reportInfo(logger_);
    timeLog("init");
}

void MLFMA::reportInfo(std::ostream& strm) const
{
    EM::reportInfo(strm);
    strm << "MLFMA Level Information\n    Number of level: " << levels_ + 1 << '\n';
}

void MLFMA::solve()
{
    const size_t n = unknowns_, r = n_inc_;
    check(emfa_device_alloc(ctx_, 8 * n * r, &V_), ctx_, "alloc V");
    check(emfa_device_alloc(ctx_, 16 * n * r, &Ibox_), ctx_, "alloc I");
    check(emfa_device_alloc(ctx_, 16 * n * r, &I_), ctx_, "alloc I");
    check(emfa_mlfma_fill_v(ml_, inc_angles_.data(), n_inc_, V_, nullptr), ctx_, "fillVbyBox");
    timeLog("fillVbyBox");
    emfa_solver_params_t sp{EMFA_BICGSTAB, 30, max_iter_, tol_, 0, EMFA_MV_AUTO, 0, 0};
    emfa_solve_info_t info{};
    emfa_status_t s = emfa_mlfma_solve(ml_, V_, n_inc_, Ibox_, &sp, &info, nullptr);
    if (s == EMFA_ERR_NOT_CONVERGED)
        logger_ << "    WARNING: Iteration cannot converge\n";
    else
        check(s, ctx_, "iterativeSolve");
    logger_ << "    Iterative number: " << info.iterations << '\n';
    std::cout << "    Iterative number: " << info.iterations << std::endl;
    check(emfa_mlfma_unpermute(ml_, Ibox_, n_inc_, I_, nullptr), ctx_, "unpermute");
    timeLog("iterativeSolve");
}

void MLFMA::output()
{
    emfa_fill_params_t fp{EMFA_CFIE, EMFA_F32, (double)incidence_.freq, (double)alpha_, 0, 0, 0};
    if (rtype_ == policy::MonoRCS) {
        writeMonostatic(fp, I_);
        timeLog("getMonostaticRCS");
    } else {
        writeBistatic(fp, I_);
        timeLog("getBistaticRCS");
    }
}

void MLFMA::clear()
{
    for (void* p : {V_, Ibox_, I_})
        if (p) emfa_device_free(ctx_, p);
    V_ = Ibox_ = I_ = nullptr;
    if (ml_) emfa_mlfma_destroy(ml_);
    ml_ = nullptr;
    EM::clear();
}

}  // namespace mom

namespace solver {

template <typename S>
static void invoke_solver(component::ConfigLoader* ploader)
{
    auto s = std::make_unique<S>();
    s->init(ploader);
    s->reportInfo(std::cout);
    s->solve();
    s->output();
    s->clear();
}

void loadSolver(const std::string& conf_file)
{
    component::ConfigLoader loader;
    loader.load(conf_file);
    std::string type = loader.getSolverType();
    if (type == "EFIE")
        invoke_solver<mom::EFIE>(&loader);
    else if (type == "CFIE")
        invoke_solver<mom::CFIE>(&loader);
    else if (type == "MLFMA")
        invoke_solver<mom::MLFMA>(&loader);
    else
        throw component::ConfigInvalid("undefined EM solver type (" + type + ')');
}

}  // namespace solver

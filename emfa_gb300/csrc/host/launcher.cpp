// emfa_launcher: drop-in for EMLauncher (EMLauncher/launcher.cpp:8-49).
// Reads the config path from stdin (or argv[1]), runs solver::loadSolver and
// maps exceptions to the reference's exit-state strings.
//   emfa_launcher --check-config <path>   parse only (no GPU), print the values
#include <iostream>
#include <string>

#include "emfa_host.h"

static int check_config(const std::string& path)
{
    component::ConfigLoader l;
    l.load(path);
    auto inc = l.getInc();
    auto sca = l.getSca();
    auto sig = l.getSigma();
    std::cout << "{\"solver\": \"" << l.getSolverType() << "\", \"freq\": " << inc.freq << ", \"theta\": " << inc.theta
              << ", \"phi\": " << inc.phi << ", \"pole\": " << inc.pole << ", \"theta_from\": " << sca.theta_from
              << ", \"theta_to\": " << sca.theta_to << ", \"phi_from\": " << sca.phi_from
              << ", \"alpha\": " << l.getAlpha() << ", \"sigma\": [" << sig.real() << ", " << sig.imag()
              << "], \"mesh\": \"" << l.getMeshPath() << "\", \"precond\": " << (l.getPreconditioningSwitch() ? 1 : 0)
              << ", \"box\": " << l.getMLFMABoxThreshold() << ", \"tol\": " << l.getIterationThreshold()
              << ", \"maxit\": " << l.getMaxIterationNum() << ", \"gpu_precision\": \""
              << l.getGpu("gpu_precision:", "f32") << "\"}" << std::endl;
    return 0;
}

int main(int argc, char** argv)
{
    std::string config, state("OK");
    if (argc > 2 && std::string(argv[1]) == "--check-config") {
        try {
            return check_config(argv[2]);
        } catch (const std::exception& e) {
            std::cout << "{\"error\": \"" << e.what() << "\"}" << std::endl;
            return 2;
        }
    }
    if (argc > 1) {
        config = argv[1];
    } else {
        std::cout << "Input Path of Config File:";
        std::getline(std::cin, config);
    }
    if (config.empty()) config = "CONFIG.yml";
    try {
        solver::loadSolver(config);
    } catch (const component::ConfigInvalid& e) {
        state = std::string("[ConfigParameter Error]") + e.what();
    } catch (const component::FileError& e) {
        state = std::string("[File Error]") + e.what();
    } catch (const std::invalid_argument& e) {
        state = std::string("[InvalidArgument Error]") + e.what();
    } catch (const std::runtime_error& e) {
        state = std::string("[Runtime Error]") + e.what();
    } catch (const std::exception& e) {
        state = std::string("[Unrecognized Error]") + e.what();
    }
    std::cout << "Exit State: " << state << std::endl;
    return state == "OK" ? 0 : 1;
}

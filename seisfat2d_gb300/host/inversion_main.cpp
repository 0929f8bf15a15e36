// inversion.exe parameters.txt — the reference's tomography driver
// (src/inversion_main.cpp:4-41) on the GB300 engine. The reference reads
// `inversion_type`, which run/parameters.txt spells `inv_type`; both are
// accepted: 0 isotropic (Tomography_ISO), 1 anisotropic VTI (Tomography_VTI).
#include <chrono>
#include <iostream>

#include "admin.hpp"
#include "inversion.hpp"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: inversion.exe parameters.txt\n";
        return 1;
    }
    try {
        auto file = std::string(argv[1]);
        std::string t = catch_parameter("inversion_type", file);
        if (t.empty()) t = catch_parameter("inv_type", file);
        const int type = t.empty() ? 0 : std::stoi(t);
        if (type != 0 && type != 1) throw std::invalid_argument("inv_type must be 0 (isotropic) or 1 (VTI)");
        Inversion* inv = (type == 1) ? (Inversion*)new Tomography_VTI() : (Inversion*)new Tomography_ISO();
        inv->parameters = file;
        inv->set_parameters();
        inv->import_obsData();
        auto ti = std::chrono::system_clock::now();
        while (true) {
            inv->forward_modeling();
            inv->check_convergence();
            if (inv->converged) break;
            inv->optimization();
            inv->model_update();
        }
        auto tf = std::chrono::system_clock::now();
        inv->export_results();
        std::chrono::duration<double> elapsed = tf - ti;
        std::cout << "\nRun time: " << elapsed.count() << " s." << std::endl;
        delete inv;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    return 0;
}

// modeling.exe parameters.txt — the reference's modeling driver
// (src/modeling_main.cpp:4-36) on the GB300 engine. Same inputs, same output
// files (<modeling_output_folder><modeling_type>_nStations<nrec>_shot_<k>.bin).
// With `batch_shots = true` in parameters.txt all shots run in one persistent
// launch (sf_batch_forward) instead of the per-shot loop; the files are the
// same.
#include <chrono>
#include <iostream>
#include <vector>

#include "admin.hpp"
#include "modeling.hpp"

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: modeling.exe parameters.txt\n";
        return 1;
    }
    try {
        std::vector<Modeling*> modeling = {new Eikonal_ISO(), new Eikonal_ANI()};
        auto file = std::string(argv[1]);
        auto type = std::stoi(catch_parameter("modeling_type", file));
        Modeling* m = modeling.at(type);
        m->parameters = file;
        m->set_parameters();
        const bool batched = str2bool(catch_parameter("batch_shots", file));
        const bool quiet = str2bool(catch_parameter("quiet", file));

        auto ti = std::chrono::system_clock::now();
        if (!batched) {
            for (int shot = 0; shot < m->geometry->nsrc; shot++) {
                m->srcId = shot;
                m->set_shot_point();
                if (!quiet) m->show_information();
                m->time_propagation();
                m->export_seismogram();
            }
        } else {
            const int ns = m->geometry->nsrc, nr = m->geometry->nrec;
            std::vector<sf_shot> shots(ns);
            for (int s = 0; s < ns; s++) shots[s] = {m->geometry->xsrc[s], m->geometry->zsrc[s], 0, 0};
            std::vector<float> picks((size_t)ns * nr);
            sf_check(sf_batch_forward(m->engine(), m->anisotropic(), shots.data(), ns, m->geometry->xrec,
                                      m->geometry->zrec, nr, picks.data(), SF_MEM_HOST, 0, nullptr),
                     m->engine(), "sf_batch_forward");
            for (int s = 0; s < ns; s++) {
                std::string f = m->data_folder + m->modeling_type + "_nStations" + std::to_string(nr) + "_shot_" +
                                std::to_string(s + 1) + ".bin";
                export_binary_float(f, picks.data() + (size_t)s * nr, nr);
            }
        }
        auto tf = std::chrono::system_clock::now();
        std::chrono::duration<double> elapsed = tf - ti;
        std::cout << "\nRun time: " << elapsed.count() << " s." << std::endl;
        for (auto* p : modeling) delete p;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    return 0;
}

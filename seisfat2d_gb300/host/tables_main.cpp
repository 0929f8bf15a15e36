// traveltime_tables.exe parameters.txt — the traveltime tables of the
// reference's Kirchhoff migration (Migration::set_src_travel_times /
// set_rec_travel_times, src/migration/migration.cu:116-171): one full padded
// traveltime field per source and per receiver, written as
// <mig_tables_folder>eikonal_src_<k>.bin and eikonal_rec_<k>.bin (nzz x nxx
// floats, z fastest). Here every table is solved in one batched launch per
// group instead of one launch sequence and one device-to-host copy per table.
// `anisotropy = true` selects the anisotropic solve (migration.cu:29-30).
#include <iostream>
#include <vector>

#include "admin.hpp"
#include "modeling.hpp"

static void write_tables(Modeling* m, const float* x, const float* z, int n, const std::string& prefix)
{
    const int chunk = 256;  // tables kept on the device per launch
    std::vector<float> table((size_t)m->matsize);
    for (int first = 0; first < n; first += chunk) {
        const int cnt = std::min(chunk, n - first);
        std::vector<sf_shot> shots(cnt);
        for (int k = 0; k < cnt; k++) shots[k] = {x[first + k], z[first + k], 0, 0};
        sf_check(sf_batch_forward(m->engine(), m->anisotropic(), shots.data(), cnt, nullptr, nullptr, 0, nullptr,
                                  SF_MEM_HOST, SF_KEEP_TABLES, nullptr),
                 m->engine(), "sf_batch_forward");
        for (int k = 0; k < cnt; k++) {
            sf_check(sf_batch_table(m->engine(), k, table.data(), SF_MEM_HOST, nullptr), m->engine(), "sf_batch_table");
            export_binary_float(prefix + std::to_string(first + k + 1) + ".bin", table.data(), m->matsize);
        }
    }
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: traveltime_tables.exe parameters.txt\n";
        return 1;
    }
    try {
        std::string file = argv[1];
        Modeling* m = str2bool(catch_parameter("anisotropy", file)) ? (Modeling*)new Eikonal_ANI()
                                                                     : (Modeling*)new Eikonal_ISO();
        m->parameters = file;
        m->set_parameters();
        std::string folder = catch_parameter("mig_tables_folder", file);
        write_tables(m, m->geometry->xsrc, m->geometry->zsrc, m->geometry->nsrc, folder + "eikonal_src_");
        write_tables(m, m->geometry->xrec, m->geometry->zrec, m->geometry->nrec, folder + "eikonal_rec_");
        delete m;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    return 0;
}

#include "geometry.hpp"

#include <vector>

#include "admin.hpp"

void Geometry::set_parameters()
{
    std::vector<std::string> SPS, RPS;
    import_text_file(catch_parameter("SPS", parameters), SPS);
    import_text_file(catch_parameter("RPS", parameters), RPS);
    nsrc = (int)SPS.size();
    nrec = (int)RPS.size();
    delete[] xsrc; delete[] zsrc; delete[] xrec; delete[] zrec;
    xsrc = new float[nsrc]();
    zsrc = new float[nsrc]();
    xrec = new float[nrec]();
    zrec = new float[nrec]();
    for (int i = 0; i < nsrc; i++) {
        std::vector<std::string> aux = split(SPS[i], ',');
        xsrc[i] = std::stof(aux.at(0));
        zsrc[i] = std::stof(aux.at(1));
    }
    for (int i = 0; i < nrec; i++) {
        std::vector<std::string> aux = split(RPS[i], ',');
        xrec[i] = std::stof(aux.at(0));
        zrec[i] = std::stof(aux.at(1));
    }
}

Geometry::~Geometry()
{
    delete[] xsrc;
    delete[] zsrc;
    delete[] xrec;
    delete[] zrec;
}

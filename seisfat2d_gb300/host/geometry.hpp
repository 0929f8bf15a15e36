// Acquisition geometry (src/geometry/geometry.hpp): SPS and RPS text files,
// one "x,z" pair in metres per line.
#ifndef SF_HOST_GEOMETRY_HPP
#define SF_HOST_GEOMETRY_HPP

#include <string>

class Geometry
{
public:
    int nsrc = 0;
    int nrec = 0;

    float* xsrc = nullptr;
    float* zsrc = nullptr;

    float* xrec = nullptr;
    float* zrec = nullptr;

    std::string parameters;

    void set_parameters();  // geometry.cpp:3-42
    ~Geometry();
};

#endif

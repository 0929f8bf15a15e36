// Host utilities of the parameters.txt workflow, with the semantics of the
// reference's admin module (src/admin/admin.hpp, admin.cpp). No FFTW: the
// traveltime path never used it.
#ifndef SF_HOST_ADMIN_HPP
#define SF_HOST_ADMIN_HPP

#include <string>
#include <vector>

bool str2bool(std::string s);                          // admin.cpp:15-23 (anything but "true" is false)
void import_binary_float(std::string path, float* array, int n);   // admin.cpp:25-35
void export_binary_float(std::string path, float* array, int n);   // admin.cpp:37-49
// admin.cpp:51-63: every line not starting with '#' (empty lines are skipped
// here; the reference kept them and then failed to parse them)
void import_text_file(std::string path, std::vector<std::string>& elements);
// admin.cpp:65-100: first line (not starting with '#' or ' ') that begins
// with `target`; the value starts two characters after the first '=', ends at
// '#', and has every space removed. Missing key -> "".
std::string catch_parameter(std::string target, std::string file);
std::vector<std::string> split(std::string s, char delimiter);     // admin.cpp:102-113

// Throws std::runtime_error with the engine's message for a non-zero status.
void sf_check(int status, void* ctx, const char* what);

#endif

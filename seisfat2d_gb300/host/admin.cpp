#include "admin.hpp"

#include <algorithm>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "seisfat2d.h"

bool str2bool(std::string s)
{
    std::for_each(s.begin(), s.end(), [](char& c) { c = (char)::tolower((unsigned char)c); });
    bool b = false;
    std::istringstream(s) >> std::boolalpha >> b;
    return b;
}

void import_binary_float(std::string path, float* array, int n)
{
    std::ifstream file(path, std::ios::in | std::ios::binary);
    if (!file.is_open()) throw std::invalid_argument("Error: " + path + " could not be opened!");
    file.read((char*)array, (std::streamsize)n * sizeof(float));
}

void export_binary_float(std::string path, float* array, int n)
{
    std::ofstream file(path, std::ios::out | std::ios::binary);
    if (!file.is_open()) throw std::invalid_argument("Error: " + path + " could not be opened!");
    file.write((char*)array, (std::streamsize)n * sizeof(float));
}

void import_text_file(std::string path, std::vector<std::string>& elements)
{
    std::ifstream file(path, std::ios::in);
    if (!file.is_open()) throw std::invalid_argument("Error: " + path + " could not be opened!");
    std::string line;
    while (getline(file, line))
        if (!line.empty() && line[0] != '#') elements.push_back(line);
}

std::string catch_parameter(std::string target, std::string file)
{
    std::ifstream parameters(file);
    if (!parameters.is_open()) throw std::invalid_argument("Error: " + file + " could not be opened!");
    std::string line, variable;
    while (getline(parameters, line)) {
        if (line.empty() || line.front() == '#' || line.front() == ' ') continue;
        if (line.find(target) == 0) {
            size_t eq = line.find("=");
            size_t start = (eq == std::string::npos) ? 1 : eq + 2;
            for (size_t i = start; i < line.size(); i++) {
                if (line[i] == '#') break;
                variable += line[i];
            }
            break;
        }
    }
    variable.erase(std::remove(variable.begin(), variable.end(), ' '), variable.end());
    return variable;
}

std::vector<std::string> split(std::string s, char delimiter)
{
    std::string token;
    std::vector<std::string> tokens;
    std::istringstream ts(s);
    while (getline(ts, token, delimiter)) tokens.push_back(token);
    return tokens;
}

void sf_check(int status, void* ctx, const char* what)
{
    if (status == SF_OK) return;
    std::string msg = std::string(what) + ": " + sf_status_string(status);
    if (ctx) msg += std::string(" (") + sf_ctx_last_error((sf_ctx*)ctx) + ")";
    throw std::runtime_error(msg);
}

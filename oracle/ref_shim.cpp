// ref_shim.cpp -- link-time definitions the reference objects need from
// src/FFEA_user_info.cpp, which itself cannot be compiled without the
// configure-generated FFEA_version.h.  Only the logging globals and print
// helpers are provided; none of them is on the blob-update path.
// TEST INFRASTRUCTURE ONLY.
#include <cstdio>
#include <string>

namespace userInfo {
std::string log_out_fname = "";
int verblevel = 0;
FILE *log_out = nullptr;
}  // namespace userInfo

void set_verbosity_level(int l) { userInfo::verblevel = l; }
void set_log_fname(std::string s) { userInfo::log_out_fname = s; }
void print_normal(std::string) {}
void print_mid(std::string) {}
void print_high(std::string) {}
void print_mania(std::string) {}
void print_ffea_version(FILE *) {}
void print_ffea_compilation_details(FILE *) {}

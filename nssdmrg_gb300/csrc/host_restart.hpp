// Block restart files in the reference's text format (see host_restart.cpp).
#pragma once

#include <iosfwd>
#include <string>

#include "host_sparse.hpp"

namespace nss {

void write_block(std::ostream &os, const Block &b);
Block read_block(std::istream &is);
void save_block_file(const std::string &path, const Block &b);
Block load_block_file(const std::string &path);

}  // namespace nss

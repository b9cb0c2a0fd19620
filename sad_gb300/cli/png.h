// png.h -- PNG reading (8-bit RGB out) and writing (8-bit RGB) for the command-line host.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace sadcli {

struct Image8 {
    int width = 0, height = 0;
    bool gray = false;         // the file held a single grey channel (with or without alpha)
    std::vector<uint8_t> rgb;  // [height][width][3]
};

// Throws std::runtime_error on unreadable or unsupported files.
Image8 read_png(const std::string& path);
bool write_png(const std::string& path, const uint8_t* rgb, int width, int height);

}  // namespace sadcli

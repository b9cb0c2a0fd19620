// png.h -- image files for the command-line host: PNG reading (8-bit RGB out) and writing,
// baseline JPEG reading (jpeg.cpp).
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
Image8 read_jpeg(const std::string& path);
bool is_jpeg_file(const std::string& path);
// PNG or JPEG by the file's leading bytes (the reference host reads both through one loader).
Image8 read_image(const std::string& path);

}  // namespace sadcli

// png_check.cpp -- test driver for the command-line host's PNG codec (sad_gb300/cli/png.cpp).
//   png_check read <in.png> <out.raw>           writes "w h gray\n" then the RGB bytes
//   png_check write <in.raw> <w> <h> <out.png>  raw RGB bytes -> PNG
// Exit 0 on success, 1 with the decoder's message on stderr otherwise.
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "png.h"

int main(int argc, char** argv) {
    try {
        std::string mode = argc > 1 ? argv[1] : "";
        if (mode == "read" && argc == 4) {
            sadcli::Image8 img = sadcli::read_image(argv[2]);
            std::FILE* f = std::fopen(argv[3], "wb");
            if (!f) return 1;
            std::fprintf(f, "%d %d %d\n", img.width, img.height, img.gray ? 1 : 0);
            std::fwrite(img.rgb.data(), 1, img.rgb.size(), f);
            return std::fclose(f) == 0 ? 0 : 1;
        }
        if (mode == "write" && argc == 6) {
            std::ifstream in(argv[2], std::ios::binary);
            std::vector<unsigned char> rgb((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
            int w = std::atoi(argv[3]), h = std::atoi(argv[4]);
            if (rgb.size() != size_t(w) * h * 3) return 1;
            return sadcli::write_png(argv[5], rgb.data(), w, h) ? 0 : 1;
        }
        std::fprintf(stderr, "usage: png_check read <in.png> <out.raw> | write <in.raw> <w> <h> <out.png>\n");
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
}

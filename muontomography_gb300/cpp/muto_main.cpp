// Command-line program (the reference's MuToTest.cpp:15-83): reads a JSON
// config, loads the raw-hit data files, reconstructs with the method whose
// key is present ("poca", "mlsd", "map", "slr", "slr_iter" or "pocut") on the GPU and writes the image.
//
// Top-level keys: data_files, detector_height, detector_middle, output_file;
// optional data_precision (4 = float32 records, the default; 8 = float64).
#include <chrono>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "MutoConfig.h"
#include "MutoFile.h"
#include "MutoReconstruction.h"

int main(int argc, char** argv) {
    MutoConfig config;
    const std::string path = argc > 1 ? argv[1] : "example.json";
    if (!config.loadFile(path)) {
        std::cerr << "Configuration file load error for: " << path << std::endl;
        return 1;
    }
    const auto ts = std::chrono::steady_clock::now();
    std::vector<std::string> files;
    std::vector<MTfloat> zlayers;
    int nMiddle = 0, precision = 4;
    std::string output;
    try {
        for (const json& f : config.get("data_files").items()) files.push_back(f.get_string());
        for (const json& z : config.get("detector_height").items()) zlayers.push_back(z.get_double());
        nMiddle = static_cast<int>(config.get("detector_middle").get_int());
        output = config.get("output_file").get_string();
        if (config.exist("data_precision")) precision = static_cast<int>(config.get("data_precision").get_int());
    } catch (const std::exception& e) {
        std::cerr << "Configuration error: " << e.what() << std::endl;
        return 1;
    }
    MutoMuonData data = MutoFile::getMuonData(files, zlayers, nMiddle, precision);

    std::unique_ptr<MutoGpuReconstruction> rec;
    std::string method;
    ImageHeader header;
    auto iterations = [&](const char* key) {
        const json& m = config.get(key);
        return m.contains("num_iteration") ? static_cast<MTindex>(m.at("num_iteration").get_int()) : 10u;
    };
    if (config.exist("poca")) {
        method = "poca";
        rec.reset(new MutoPoCA(config.get("poca")));
        header.nIter = 1;
    } else if (config.exist("mlsd")) {
        method = "mlsd";
        rec.reset(new MutoMLSD(config.get("mlsd")));
        header.nIter = iterations("mlsd");
    } else if (config.exist("map")) {
        method = "map";
        rec.reset(new MutoMAP(config.get("map")));
        header.nIter = iterations("map");
    } else if (config.exist("slr")) {
        method = "slr";
        rec.reset(new MutoSLR(config.get("slr")));
        header.nIter = 1;
    } else if (config.exist("slr_iter")) {
        method = "slr_iter";
        rec.reset(new MutoSLRIter(config.get("slr_iter")));
        header.nIter = 1;
    } else if (config.exist("pocut")) {
        method = "pocut";
        rec.reset(new MutoPoCut(config.get("pocut")));
        header.nIter = 1;
    } else {
        std::cerr << "No supported reconstruction key (poca, mlsd, map, slr, slr_iter, pocut) in " << path
                  << std::endl;
        return 1;
    }
    if (!rec->ok()) return 1;
    header.grid = rec->getCurrentGrid();
    Image img = rec->reconstruct(data);
    if (img.size() == 0) return 1;
    header.fPrecision = 4;
    header.method = method;
    header.nRay = static_cast<MTindex>(data.size());
    if (!MutoFile::saveImage(img, header, output)) return 1;
    const auto span = std::chrono::duration_cast<std::chrono::duration<double>>(std::chrono::steady_clock::now() - ts);
    std::cout << "Reconstruction with <" << method << "> took: " << span.count() << " seconds. " << std::endl;
    return 0;
}

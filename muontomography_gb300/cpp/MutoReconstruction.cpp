// Reconstruction classes over the C ABI.  See MutoReconstruction.h.
#include "MutoReconstruction.h"

#include <iostream>

#include "MutoFile.h"

namespace {
json empty_object() { return json::parse("{}"); }
}  // namespace

MutoGpuReconstruction::MutoGpuReconstruction(const char* method, const json& config)
    : fConfig(config), fMethod(method) {
    const std::string text = config.is_object() ? config.dump() : std::string("{}");
    try {
        fLogPrint = config.is_object() && config.value("log_results", false);
    } catch (const std::exception&) {
        fLogPrint = false;
    }
    const int rc = muto_create(method, text.c_str(), &fHandle);
    if (rc != MUTO_OK) {
        std::cerr << "Error: cannot create the " << method << " reconstruction (code " << rc << ")" << std::endl;
        fHandle = nullptr;
    }
}

MutoGpuReconstruction::~MutoGpuReconstruction() {
    if (fHandle) muto_destroy(fHandle);
}

VoxelGrid MutoGpuReconstruction::getCurrentGrid() const {
    muto_grid g{};
    if (fHandle) muto_get_grid(fHandle, &g);
    return VoxelGrid{g.nx, g.ny, g.nz, g.x_min, g.y_min, g.z_min, g.dx, g.dy, g.dz};
}

muto_status MutoGpuReconstruction::status() const {
    muto_status s{};
    if (fHandle) muto_get_status(fHandle, &s);
    return s;
}

bool MutoGpuReconstruction::check(int rc, const char* what) {
    if (rc == MUTO_OK) return true;
    std::cerr << "Error in " << what << ": " << status().message << std::endl;
    return false;
}

void MutoGpuReconstruction::logMessage(const std::string& msg, bool printTime) {
    if (!fLogPrint) return;
    std::cout << msg;
    if (printTime) {
        const auto span =
            std::chrono::duration_cast<std::chrono::duration<double>>(std::chrono::steady_clock::now() - fTimeStart);
        std::cout << " Time: " << span.count() << " seconds. ";
    }
    std::cout << std::endl;
}

Image MutoGpuReconstruction::fetchImage() {
    const VoxelGrid g = getCurrentGrid();
    Image img(g.nx, g.ny, g.nz);
    if (!check(muto_get_image(fHandle, img.data(), static_cast<uint64_t>(img.size())), "muto_get_image")) return Image{};
    return img;
}

// ---------------------------------------------------------------------------
MutoPoCA::MutoPoCA() : MutoGpuReconstruction("poca", empty_object()) {}
MutoPoCA::MutoPoCA(json config) : MutoGpuReconstruction("poca", config) {}
MutoPoCA::MutoPoCA(const char* method, json config) : MutoGpuReconstruction(method, config) {}

MutoPoCut::MutoPoCut() : MutoPoCA("pocut", empty_object()) {}
MutoPoCut::MutoPoCut(json config) : MutoPoCA("pocut", config) {}

MutoSLR::MutoSLR() : MutoGpuReconstruction("slr", empty_object()) {}
MutoSLR::MutoSLR(json config) : MutoGpuReconstruction("slr", config) {}
MutoSLR::MutoSLR(const char* method, json config) : MutoGpuReconstruction(method, config) {}

MutoSLRIter::MutoSLRIter() : MutoSLR("slr_iter", empty_object()) {}
MutoSLRIter::MutoSLRIter(json config) : MutoSLR("slr_iter", config) {}

Image MutoPoCA::reconstruct(const MutoMuonData& rays) { return reconstructOnce(rays); }
Image MutoSLR::reconstruct(const MutoMuonData& rays) { return reconstructOnce(rays); }

// the one-shot methods (PoCA, PoCut, SLR, SLRIter): the image comes out of prepare
Image MutoGpuReconstruction::reconstructOnce(const MutoMuonData& rays) {
    if (!fHandle) return Image{};
    fTimeStart = std::chrono::steady_clock::now();
    const muto_ray* r = rays.empty() ? nullptr : reinterpret_cast<const muto_ray*>(rays.data());
    if (!check(muto_load_tracks(fHandle, r, rays.size(), 0), "muto_load_tracks")) return Image{};
    if (!check(muto_prepare(fHandle), "muto_prepare")) return Image{};
    if (fLogPrint) {  // logResults, src/MutoPoCA.cpp:176-183
        const muto_status s = status();
        const bool slr = fMethod.compare(0, 3, "slr") == 0;  // src/MutoSLR.cpp:111-116
        std::cout << "==================================================" << std::endl;
        std::cout << (slr ? "|| SLR reconstruction results                  ||"
                          : "|| PoCA reconstruction results                  ||")
                  << std::endl;
        std::cout << "==================================================" << std::endl;
        std::cout << "number of rays processed: " << s.n_total << std::endl;
        if (!slr) {
            std::cout << "number of unparalleled rays: " << s.n_not_parallel << std::endl;
            std::cout << "number of interactions in voxels: " << s.n_scat_in_grid << std::endl;
        }
    }
    return fetchImage();
}

// ---------------------------------------------------------------------------
MutoMLSD::MutoMLSD() : MutoMLSD("mlsd", empty_object()) {}
MutoMLSD::MutoMLSD(json config) : MutoMLSD("mlsd", config) {}
MutoMLSD::MutoMLSD(const char* method, json config) : MutoGpuReconstruction(method, config) {
    try {
        if (config.is_object()) fNIteration = config.value("num_iteration", 10);
    } catch (const std::exception&) {
    }
}

Image MutoMLSD::reconstruct(const MutoMuonData& rays) {
    if (!fHandle) return Image{};
    fTimeStart = std::chrono::steady_clock::now();
    logMessage("==================================================");
    logMessage("|| MLSD reconstruction start                    ||");
    logMessage("==================================================");
    // initial image, src/MutoMLSD.cpp:226-266: method 0 reads initial_image_file
    int method = 0;
    std::string file;
    try {
        method = fConfig.value("initialize_method", 0);
        file = fConfig.value("initial_image_file", "");
    } catch (const std::exception&) {
    }
    if (method == 0) {
        auto ih = MutoFile::loadImage(file);
        if (ih.first.size() == 0) {
            std::cout << "Warning: Initial image file <" << file << "> not exist. " << std::endl;
            std::cout << "\tSetting initialization method to random numbers ..." << std::endl;
            if (!check(muto_set_initial_image(fHandle, nullptr, nullptr), "muto_set_initial_image")) return Image{};
        } else {
            const VoxelGrid cur = getCurrentGrid();
            const VoxelGrid& in = ih.second.grid;
            if (in.nx != cur.nx || in.ny != cur.ny || in.nz != cur.nz) {
                std::cout << "Warning: Initial image's dimensions do not match the configuration. " << std::endl;
                std::cout << "\tResetting grid configuration as defined in input image  ..." << std::endl;
            }
            const muto_grid g{in.nx, in.ny, in.nz, 0, in.x_min, in.y_min, in.z_min, in.dx, in.dy, in.dz};
            if (!check(muto_set_initial_image(fHandle, ih.first.data(), &g), "muto_set_initial_image")) return Image{};
        }
    }
    logMessage("Initial image was loaded / generated.", true);
    const muto_ray* r = rays.empty() ? nullptr : reinterpret_cast<const muto_ray*>(rays.data());
    if (!check(muto_load_tracks(fHandle, r, rays.size(), 0), "muto_load_tracks")) return Image{};
    if (!check(muto_prepare(fHandle), "muto_prepare")) return Image{};
    logMessage("Weight matrix was generated.", true);
    logMessage("\nStart EM iteration to find the Maximum Likelihood ... ");
    if (!fLogPrint) {
        if (!check(muto_iterate(fHandle, fNIteration), "muto_iterate")) return Image{};
    } else {
        for (int it = 0; it < fNIteration; ++it) {
            if (!check(muto_iterate(fHandle, 1), "muto_iterate")) return Image{};
            const muto_status s = status();
            if (s.iterations_done <= it) break;  // early stop
            logMessage("Iteration #" + std::to_string(it) + " finished. ", true);
            logMessage("\tcost function = " + std::to_string(s.cost));
            if (s.early_stopped) {
                logMessage("Early stop at iteration#" + std::to_string(it) +
                           ". Minimum cost function = " + std::to_string(s.cost_prev));
                break;
            }
        }
        const muto_status s = status();  // logResults, src/MutoMLSD.cpp:535-543
        std::cout << std::endl << "==================================================" << std::endl;
        std::cout << "|| MLSD reconstruction results                  ||" << std::endl;
        std::cout << "==================================================" << std::endl;
        std::cout << "number of rays processed: " << s.n_total << std::endl;
        std::cout << "number of interactions in voxels: " << s.n_scat_in_grid << std::endl;
        std::cout << "number of iterations: " << fNIteration << std::endl;
    }
    return fetchImage();
}

// ---------------------------------------------------------------------------
MutoMAP::MutoMAP() : MutoMLSD("map", empty_object()) {}
MutoMAP::MutoMAP(json config) : MutoMLSD("map", config) {}

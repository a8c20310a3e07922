// core_geometry.cpp - VoxelGrid and ComputationalDomain of the MIDSX C++ API.
// Reference: src/MIDSX/Core/voxel_grid.cpp, src/MIDSX/Core/computational_domain.cpp.
// The reference loads NIfTI through an embedded Python interpreter and nibabel and parses
// the scene with nlohmann/json; here both are read by small readers written for this file
// format (NIfTI-1 single file: 348-byte header, data at vox_offset) and this JSON schema.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <unordered_set>
#include <vector>

#if defined(__has_include) && !defined(MIDSX_NO_ZLIB)
#if __has_include(<zlib.h>)
#include <zlib.h>
#define MIDSX_HAVE_ZLIB 1
#endif
#endif

#include "MIDSX/Core/computational_domain.h"

namespace {

std::vector<unsigned char> read_file_bytes(const std::string& path) {
    bool gz = path.size() > 3 && path.compare(path.size() - 3, 3, ".gz") == 0;
    std::vector<unsigned char> out;
    if (gz) {
#ifdef MIDSX_HAVE_ZLIB
        gzFile f = gzopen(path.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + path);
        unsigned char buf[1 << 16];
        int n;
        while ((n = gzread(f, buf, sizeof(buf))) > 0) out.insert(out.end(), buf, buf + n);
        gzclose(f);
        if (n < 0) throw std::runtime_error("gzip error reading " + path);
#else
        throw std::runtime_error("this build has no zlib: decompress " + path + " to .nii first");
#endif
    } else {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error("cannot open " + path);
        out.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    return out;
}

template <typename T>
T rd(const std::vector<unsigned char>& b, size_t off) {
    T v;
    std::memcpy(&v, b.data() + off, sizeof(T));
    return v;
}

// ------------------------------------------------------------------ tiny JSON ------
struct JVal {
    enum Kind { Null, Num, Str, Arr, Obj } kind = Null;
    double num = 0;
    std::string str;
    std::vector<JVal> arr;
    std::map<std::string, JVal> obj;
    const JVal& at(const std::string& k) const {
        auto it = obj.find(k);
        if (it == obj.end()) throw std::runtime_error("JSON key missing: " + k);
        return it->second;
    }
};

struct JParser {
    const std::string& s;
    size_t i = 0;
    void ws() {
        while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
    }
    JVal parse() {
        ws();
        if (i >= s.size()) throw std::runtime_error("JSON: unexpected end");
        char c = s[i];
        JVal v;
        if (c == '{') {
            v.kind = JVal::Obj;
            ++i;
            ws();
            if (s[i] == '}') {
                ++i;
                return v;
            }
            for (;;) {
                ws();
                JVal k = parse();
                ws();
                if (s[i++] != ':') throw std::runtime_error("JSON: expected ':'");
                v.obj[k.str] = parse();
                ws();
                if (s[i] == ',') {
                    ++i;
                    continue;
                }
                if (s[i++] != '}') throw std::runtime_error("JSON: expected '}'");
                return v;
            }
        }
        if (c == '[') {
            v.kind = JVal::Arr;
            ++i;
            ws();
            if (s[i] == ']') {
                ++i;
                return v;
            }
            for (;;) {
                v.arr.push_back(parse());
                ws();
                if (s[i] == ',') {
                    ++i;
                    continue;
                }
                if (s[i++] != ']') throw std::runtime_error("JSON: expected ']'");
                return v;
            }
        }
        if (c == '"') {
            v.kind = JVal::Str;
            ++i;
            while (i < s.size() && s[i] != '"') {
                if (s[i] == '\\' && i + 1 < s.size()) ++i;
                v.str.push_back(s[i++]);
            }
            ++i;
            return v;
        }
        if (s.compare(i, 4, "null") == 0) {
            i += 4;
            return v;
        }
        size_t end = i;
        while (end < s.size() && (std::isdigit(static_cast<unsigned char>(s[end])) || s[end] == '-' ||
                                  s[end] == '+' || s[end] == '.' || s[end] == 'e' || s[end] == 'E'))
            ++end;
        if (end == i) throw std::runtime_error("JSON: unexpected character");
        v.kind = JVal::Num;
        v.num = std::stod(s.substr(i, end - i));
        i = end;
        return v;
    }
};

Vec3 jvec3(const JVal& v) {
    if (v.kind != JVal::Arr || v.arr.size() != 3) throw std::runtime_error("JSON: expected a 3-vector");
    return {v.arr[0].num, v.arr[1].num, v.arr[2].num};
}

std::string dirname_of(const std::string& p) {
    size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

}  // namespace

// ------------------------------------------------------------------- VoxelGrid ------
VoxelGrid::VoxelGrid(const std::string& filename) {
    if (filename.find(".nii") == std::string::npos) throw std::runtime_error("The file provided is not a NIFTI file.");
    std::vector<unsigned char> b = read_file_bytes(filename);
    if (b.size() < 352 || rd<int32_t>(b, 0) != 348) throw std::runtime_error("not a NIfTI-1 file: " + filename);
    int16_t dim[8];
    for (int k = 0; k < 8; ++k) dim[k] = rd<int16_t>(b, 40 + 2 * k);
    int16_t datatype = rd<int16_t>(b, 70);
    float pix[8];
    for (int k = 0; k < 8; ++k) pix[k] = rd<float>(b, 76 + 4 * k);
    size_t off = size_t(rd<float>(b, 108));
    float slope = rd<float>(b, 112), inter = rd<float>(b, 116);
    int units = b[123] & 0x07;
    // VoxelGridHelpers::covertUnitNameToCm; an unspecified unit is read as mm
    double scale = units == 1 ? 100.0 : units == 3 ? 1e-4 : 0.1;
    for (int k = 0; k < 3; ++k) {
        dim_vox_[size_t(k)] = std::max<int>(1, dim[k + 1]);
        spacing_(k) = double(pix[k + 1]) * scale;
    }
    size_t n = size_t(dim_vox_[0]) * dim_vox_[1] * dim_vox_[2];
    size_t width = datatype == 2 || datatype == 256 ? 1 : datatype == 4 || datatype == 512 ? 2
                   : datatype == 8 || datatype == 16 ? 4 : datatype == 64 ? 8 : 0;
    if (!width) throw std::runtime_error("unsupported NIfTI datatype");
    if (b.size() < off + n * width) throw std::runtime_error("truncated NIfTI data: " + filename);
    voxels_.resize(n);
    for (size_t i = 0; i < n; ++i) {
        double v;
        const size_t p = off + i * width;
        switch (datatype) {
            case 2: v = b[p]; break;
            case 256: v = double(int8_t(b[p])); break;
            case 4: v = rd<int16_t>(b, p); break;
            case 512: v = rd<uint16_t>(b, p); break;
            case 8: v = rd<int32_t>(b, p); break;
            case 16: v = rd<float>(b, p); break;
            default: v = rd<double>(b, p); break;
        }
        if (slope != 0.0f && !(slope == 1.0f && inter == 0.0f)) v = v * slope + inter;
        voxels_[i].materialID = static_cast<uint8_t>(v);
    }
    dim_space_ = Vec3(dim_vox_[0] * spacing_.x(), dim_vox_[1] * spacing_.y(), dim_vox_[2] * spacing_.z());
}

VoxelGrid::VoxelGrid(const VoxelIndex& dims, const Vec3& spacing, std::vector<uint8_t> ids)
    : dim_vox_(dims), spacing_(spacing) {
    size_t n = size_t(dims[0]) * dims[1] * dims[2];
    if (ids.size() != n) throw std::invalid_argument("VoxelGrid: id array size differs from dims");
    voxels_.resize(n);
    for (size_t i = 0; i < n; ++i) voxels_[i].materialID = ids[i];
    dim_space_ = Vec3(dims[0] * spacing.x(), dims[1] * spacing.y(), dims[2] * spacing.z());
}

int VoxelGrid::voxelNumber(const VoxelIndex& i) const { return i[0] + i[1] * dim_vox_[0] + i[2] * dim_vox_[0] * dim_vox_[1]; }

Voxel& VoxelGrid::getVoxel(const VoxelIndex& i) { return voxels_.at(size_t(voxelNumber(i))); }
void VoxelGrid::setVoxel(const VoxelIndex& i, Voxel& value) { voxels_.at(size_t(voxelNumber(i))) = value; }

Vec3 VoxelGrid::getVoxelPosition(const VoxelIndex& i) const {
    return {i[0] * spacing_.x(), i[1] * spacing_.y(), i[2] * spacing_.z()};
}

bool VoxelGrid::withinGrid(const Vec3& p) const {
    return p.x() >= 0 && p.y() >= 0 && p.z() >= 0 && p.x() <= dim_space_.x() && p.y() <= dim_space_.y() &&
           p.z() <= dim_space_.z();
}

VoxelIndex VoxelGrid::getVoxelIndex(const Vec3& p) const {
    if (!withinGrid(p)) throw std::out_of_range("VoxelGrid::handleOutOfBounds: voxel index out of range");
    return {{int(p.x() / spacing_.x()), int(p.y() / spacing_.y()), int(p.z() / spacing_.z())}};
}

std::vector<int> VoxelGrid::getMaterialIds() const {
    std::set<int> s;
    for (auto& v : voxels_) s.insert(v.materialID);
    return {s.begin(), s.end()};
}

std::vector<std::string> VoxelGrid::getMaterialNames() const {
    InteractionData helper({});
    std::vector<std::string> out;
    for (int id : getMaterialIds()) out.push_back(helper.getAnyMaterialNameFromId(id));
    return out;
}

std::vector<uint8_t> VoxelGrid::getMaterialIdArray() const {
    std::vector<uint8_t> ids(voxels_.size());
    for (size_t i = 0; i < ids.size(); ++i) ids[i] = voxels_[i].materialID;
    return ids;
}

double VoxelGrid::getTotalEnergyDeposited() {
    double s = 0;
    for (auto& v : voxels_) s += v.dose.getSum();
    return s;
}

std::unordered_map<int, VectorValue> VoxelGrid::getEnergyDepositedInMaterials() {
    std::unordered_map<int, VectorValue> out;
    for (auto& v : voxels_) {
        VectorValue& acc = out[v.materialID];
        acc = acc + v.dose;
    }
    return out;
}

// --------------------------------------------------------- ComputationalDomain ------
ComputationalDomain::ComputationalDomain(const std::string& json_file_path, bool) {
    if (json_file_path.find(".json") == std::string::npos)
        throw std::runtime_error("The file provided is not a JSON file.");
    std::ifstream f(json_file_path);
    if (!f) throw std::runtime_error("JSON file does not exist or is not accessible.");
    std::stringstream ss;
    ss << f.rdbuf();
    std::string text = ss.str();
    JVal root;
    try {
        JParser p{text};
        root = p.parse();
    } catch (const std::exception& e) {
        throw std::runtime_error(std::string("Error parsing JSON file: ") + e.what());
    }
    dim_space_ = jvec3(root.at("dim_space"));
    InteractionData helper({});
    background_voxel.materialID = helper.getAnyMaterialIdFromName(root.at("background_material_name").str);
    std::string dir = dirname_of(json_file_path);
    for (auto& g : root.at("voxel_grids").arr) {
        std::string path = g.at("file_path").str;
        if (path.find(".nii") == std::string::npos) throw std::runtime_error("The file provided is not a NIFTI file.");
        if (path.empty() || path[0] != '/') path = dir + "/" + path;
        voxel_grids_.emplace_back(VoxelGrid(path), jvec3(g.at("origin")));
    }
}

ComputationalDomain::ComputationalDomain(const Vec3& dim_space, const std::string& background_material_name,
                                         std::vector<std::pair<VoxelGrid, Vec3>> voxel_grids)
    : voxel_grids_(std::move(voxel_grids)), dim_space_(dim_space) {
    InteractionData helper({});
    background_voxel.materialID = helper.getAnyMaterialIdFromName(background_material_name);
}

bool ComputationalDomain::isInComputationalDomain(const Vec3& p) const {
    return p.x() >= 0 && p.x() <= dim_space_.x() && p.y() >= 0 && p.y() <= dim_space_.y() && p.z() >= 0 &&
           p.z() <= dim_space_.z();
}

Voxel& ComputationalDomain::getVoxel(const Vec3& position) {
    for (auto& g : voxel_grids_) {
        Vec3 q = position - g.second;
        if (g.first.withinGrid(q)) return g.first.getVoxel(g.first.getVoxelIndex(q));
    }
    return background_voxel;
}

std::string ComputationalDomain::getBackgroundMaterialName() const {
    InteractionData helper({});
    return helper.getAnyMaterialNameFromId(background_voxel.materialID);
}

std::vector<std::string> ComputationalDomain::getMaterialNames() const {
    std::vector<std::string> names{getBackgroundMaterialName()};
    for (auto& g : voxel_grids_)
        for (auto& n : g.first.getMaterialNames())
            if (std::find(names.begin(), names.end(), n) == names.end()) names.push_back(n);
    return names;
}

InteractionData ComputationalDomain::getInteractionData() const { return InteractionData(getMaterialNames()); }

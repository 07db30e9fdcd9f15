// ref_parameter.cpp - definitions of nav24's Parameter tree members (declared in the reference's own
// core/tools/parameters/Parameter.hpp) for the reference-pin build (TEST INFRASTRUCTURE).
//
// Why not the reference's Parameter.cpp: it calls std::map::contains (C++20), while Parameter.hpp
// declares constructors with template-ids (`ParamType<T>(...)`), which g++ 13 rejects in C++20
// mode.  So the reference-pin build compiles in C++17 and takes these definitions instead: the
// same tree semantics (children by key, '/'-separated key paths, find_param = read + cast), enough
// for Calibration's constructor to find its intrinsics, distortion type and coefficients.  None of
// the BA arithmetic that the pin checks is in this file.
#include <sstream>

#include "Parameter.hpp"

namespace NAV24 {

Parameter::Parameter(const std::string& name_, const ParamPtr& parent_)
    : name(name_), type(NodeType::DEFAULT), parent(parent_) {}

Parameter::Parameter(const std::string& name_, const ParamPtr& parent_, NodeType type_) : Parameter(name_, parent_) {
    type = type_;
}

ParamPtr Parameter::getChild(const std::string& key) {
    const auto it = children.find(key);
    return it == children.end() ? ParamPtr() : it->second.lock();
}

ParamPtr Parameter::read(const std::string& key) {
    std::vector<std::string> keys;
    splitKey(keys, key);
    ParamPtr node;
    for (size_t i = 0; i < keys.size(); ++i) {
        node = i == 0 ? getChild(keys[i]) : node->getChild(keys[i]);
        if (!node) break;
    }
    return node;
}

void Parameter::insertChild(const std::string& key, const ParamPtr& child) {
    if (key.empty()) return;
    if (children.find(key) == children.end()) vChildKeys.push_back(key);
    children[key] = child;
}

void Parameter::removeChild(const std::string& key) { children.erase(key); }

void Parameter::splitKey(std::vector<std::string>& keys, const std::string& key, const std::string& delim) {
    size_t start = 0;
    for (;;) {
        const size_t pos = key.find(delim, start);
        if (pos == std::string::npos) break;
        keys.push_back(key.substr(start, pos - start));
        start = pos + delim.size();
    }
    keys.push_back(key.substr(start));
}

std::string Parameter::mergeKey(const std::vector<std::string>& keys, const std::string& delim) {
    std::string out;
    for (size_t i = 0; i < keys.size(); ++i) out += (i ? delim : std::string()) + keys[i];
    return out;
}

void Parameter::setName(const std::string& name_) {
    if (!name_.empty()) name = name_;
}

std::string Parameter::printStr(const std::string& prefix) const {
    std::ostringstream os;
    for (const auto& kv : children)
        if (auto c = kv.second.lock()) os << "\n" << prefix << kv.first << ": " << c->printStr(prefix + " ");
    return os.str();
}

template <typename T>
std::string ParamType<T>::printStr(const std::string& prefix) const {
    std::ostringstream os;
    os << (prefix.empty() ? "" : " ") << mData;
    return os.str();
}

template <typename T>
std::string ParamSeq<T>::printStr(const std::string& prefix) const {
    std::ostringstream os;
    os << (prefix.empty() ? "" : " ") << "[";
    for (size_t i = 0; i < mvData.size(); ++i) os << (i ? ", " : "") << mvData[i];
    os << "]";
    return os.str();
}

template <typename T>
std::shared_ptr<T> find_param(const std::string& tag, const ParamPtr& node) {
    if (!node) return nullptr;
    return std::dynamic_pointer_cast<T>(node->read(tag));
}

template class ParamType<std::string>;
template class ParamType<cv::Mat>;
template class ParamSeq<double>;
template std::shared_ptr<ParamType<std::string>> find_param(const std::string&, const ParamPtr&);
template std::shared_ptr<ParamType<cv::Mat>> find_param(const std::string&, const ParamPtr&);
template std::shared_ptr<ParamSeq<double>> find_param(const std::string&, const ParamPtr&);

}  // namespace NAV24

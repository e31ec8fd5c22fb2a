// yaml-cpp/yaml.h — the part of yaml-cpp's Node API the reference's description writer
// uses (Common/Util/Yaml.h, LevelSetLiquid::writeDescription), written for this project.
// TEST INFRASTRUCTURE ONLY: it lets the unmodified reference sources compile into the
// reference binary under oracle/_ref.  It stores values as strings and emits nothing.
#pragma once

#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace YAML {

enum class EmitterStyle { Default, Block, Flow };

class Node;
template <typename T> struct convert;

class Node {
public:
	Node() = default;
	template <typename T> Node(const T &v) { assign(v); }
	template <typename T> Node &operator=(const T &v) { assign(v); return *this; }
	Node &operator[](const std::string &key) {
		auto &p = map()[key];
		if (!p) p = std::make_shared<Node>();
		return *p;
	}
	Node &operator[](const char *key) { return (*this)[std::string(key)]; }
	const Node &operator[](size_t i) const { return *seq()[i]; }
	template <typename T> void push_back(const T &v) { seq().push_back(std::make_shared<Node>(Node(v))); }
	void SetStyle(EmitterStyle s) { _style = s; }
	bool IsSequence() const { return _seq != nullptr; }
	size_t size() const { return _seq ? _seq->size() : 0; }
	template <typename T> T as() const {
		T v{};
		if constexpr (requires { convert<T>::decode(*this, v); }) convert<T>::decode(*this, v);
		else { std::istringstream in(_scalar); in >> v; }
		return v;
	}
private:
	template <typename T> void assign(const T &v) {
		if constexpr (std::is_same_v<T, Node>) { _scalar = v._scalar; _seq = v._seq; _map = v._map; _style = v._style; }
		else if constexpr (requires { convert<T>::encode(v); }) *this = convert<T>::encode(v);
		else if constexpr (std::is_same_v<T, bool>) _scalar = v ? "true" : "false";
		else { std::ostringstream out; out << v; _scalar = out.str(); }
	}
	std::vector<std::shared_ptr<Node>> &seq() { if (!_seq) _seq = std::make_shared<std::vector<std::shared_ptr<Node>>>(); return *_seq; }
	const std::vector<std::shared_ptr<Node>> &seq() const { return *_seq; }
	std::map<std::string, std::shared_ptr<Node>> &map() { if (!_map) _map = std::make_shared<std::map<std::string, std::shared_ptr<Node>>>(); return *_map; }
	std::string _scalar;
	std::shared_ptr<std::vector<std::shared_ptr<Node>>> _seq;
	std::shared_ptr<std::map<std::string, std::shared_ptr<Node>>> _map;
	EmitterStyle _style = EmitterStyle::Default;
};

template <typename T> struct convert { };

}  // namespace YAML

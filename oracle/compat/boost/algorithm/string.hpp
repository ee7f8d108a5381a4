// Minimal stand-in for boost::split / boost::is_any_of, the only Boost string
// algorithms the reference's file locator names.  Test infrastructure only.
#pragma once
#include <string>
#include "string/replace.hpp"
namespace boost {
struct is_any_of_pred {
	std::string set;
	bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
inline is_any_of_pred is_any_of(const std::string& s) { return is_any_of_pred{s}; }
template <class Seq>
Seq& split(Seq& out, const std::string& in, is_any_of_pred pred) {
	out.clear();
	std::string cur;
	for (char c : in) {
		if (pred(c)) { out.push_back(cur); cur.clear(); }
		else cur.push_back(c);
	}
	out.push_back(cur);
	return out;
}
} // namespace boost

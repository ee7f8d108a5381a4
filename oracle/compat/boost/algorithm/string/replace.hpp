// Minimal stand-in for boost::replace_all, the only Boost replace algorithm the
// reference's scene registry names.  Test infrastructure only.
#pragma once
#include <string>
namespace boost {
inline void replace_all(std::string& s, const std::string& from, const std::string& to) {
	if (from.empty()) return;
	std::string::size_type pos = 0;
	while ((pos = s.find(from, pos)) != std::string::npos) {
		s.replace(pos, from.size(), to);
		pos += to.size();
	}
}
} // namespace boost

// Minimal stand-in for the one Boost.Random type the reference's radiosity
// solver names (boost::rand48).  Test infrastructure only: it lets the
// reference library be compiled from its own sources for the oracle.
//
// rand48 is the POSIX 48-bit linear congruential generator
//   x' = (0x5DEECE66D * x + 0xB) mod 2^48,  output = x' >> 17  (31 bits),
// seeded with seed(s): x = (s << 16) | 0x330E.  Constants are the published
// POSIX drand48/lrand48 ones.
#pragma once
#include <cstdint>
namespace boost {
class rand48 {
public:
	typedef std::uint32_t result_type;
	rand48() { seed(1); }
	explicit rand48(std::uint32_t s) { seed(s); }
	void seed(std::uint32_t s) { x_ = ((std::uint64_t)s << 16) | 0x330Eu; }
	static constexpr result_type min() { return 0; }
	static constexpr result_type max() { return 0x7FFFFFFFu; }
	result_type operator()() {
		x_ = (0x5DEECE66DULL * x_ + 0xBULL) & ((1ULL << 48) - 1);
		return (result_type)(x_ >> 17);
	}
private:
	std::uint64_t x_;
};
} // namespace boost

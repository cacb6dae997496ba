/* Project-written stand-in for lib/algebra/polynomial_one.hpp, which the
 * reference includes (lib/algebra/algebra.hpp:13) but does not ship.
 * Only lib/structure/s_expression.hpp:101-127 (Formula_, not on the
 * projection path) names carpio::PolynomialOne_, so this type only has to
 * exist: a sparse map from term to coefficient with an insert-or-add. */
#ifndef CARPIO_ORACLE_SHIM_POLYNOMIAL_ONE_HPP
#define CARPIO_ORACLE_SHIM_POLYNOMIAL_ONE_HPP
#include <map>
namespace carpio {
template<class COE, class TERM, class CMP = std::less<TERM> >
class PolynomialOne_ {
public:
	typedef std::map<TERM, COE, CMP> Map;
	typedef typename Map::iterator iterator;
	typedef typename Map::const_iterator const_iterator;
	void insert(const COE& c, const TERM& t) {
		iterator it = _m.find(t);
		if (it == _m.end()) { _m.insert(std::make_pair(t, c)); }
		else { it->second = it->second + c; }
	}
	iterator begin() { return _m.begin(); }
	iterator end() { return _m.end(); }
	const_iterator begin() const { return _m.begin(); }
	const_iterator end() const { return _m.end(); }
	std::size_t size() const { return _m.size(); }
protected:
	Map _m;
};
}
#endif

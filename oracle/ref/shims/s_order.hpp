/* Project-written stand-in for lib/structure/s_order.hpp, which
 * lib/structure/s_solver.hpp:11 includes but the reference does not ship.
 * Interface taken from its call sites (s_solver.hpp:77-92, 106-107, 213-217):
 * begin(), end(), next(idx), get_order(idx), size(), and construction from
 * (grid, ghost). OrderRegular_ numbers the normal cells of a regular grid in
 * the order Grid_::begin_ijk() visits them (x fastest, s_define.hpp:394-410):
 * order(i, j) = i + j * nx. The numbering only changes rounding (dot-product
 * order); the oracle restatement and the fixtures use the same numbering. */
#ifndef CARPIO_ORACLE_SHIM_S_ORDER_HPP
#define CARPIO_ORACLE_SHIM_S_ORDER_HPP
#include <memory>
namespace structure {
template<St DIM>
class Order_ {
public:
	typedef Index_<DIM> Index;
	virtual ~Order_() {}
	virtual Index begin() const = 0;
	virtual Index end() const = 0;
	virtual Index next(const Index& idx) const = 0;
	virtual St get_order(const Index& idx) const = 0;
	virtual St size() const = 0;
};

template<St DIM>
class OrderRegular_: public Order_<DIM> {
public:
	typedef Index_<DIM> Index;
	typedef std::shared_ptr<Grid_<DIM> > spGrid;
	typedef std::shared_ptr<Ghost_<DIM> > spGhost;
	OrderRegular_(spGrid g, spGhost gh) : _g(g) {
		for (St d = 0; d < 3; ++d) { _n[d] = d < DIM ? g->n(d) : 1; }
	}
	Index begin() const { return Index(0, 0, 0); }
	Index end() const {
		/* one past the last cell: the first index of row n[DIM-1] */
		Index e(0, 0, 0);
		e[DIM - 1] = _n[DIM - 1];
		return e;
	}
	Index next(const Index& idx) const {
		Index r(idx);
		for (St d = 0; d < DIM; ++d) {
			r[d] = r[d] + 1;
			if (r[d] < _n[d] || d == DIM - 1) { return r; }
			r[d] = 0;
		}
		return r;
	}
	St get_order(const Index& idx) const {
		St o = 0, s = 1;
		for (St d = 0; d < DIM; ++d) { o += St(idx[d]) * s; s *= St(_n[d]); }
		return o;
	}
	St size() const {
		St s = 1;
		for (St d = 0; d < DIM; ++d) { s *= St(_n[d]); }
		return s;
	}
protected:
	spGrid _g;
	Idx _n[3];
};
}
#endif

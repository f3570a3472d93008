// Test-infrastructure shim: the subset of boost::multi_array that the
// reference's likelihood and integral sources use (construction from
// `extents[a][b]...` or a shape array, resize that keeps the overlapping
// elements, chained operator[], data(), num_elements(), shape()).  Row-major
// storage like Boost's default.  Only used to compile the reference's own
// sources into the checker library under oracle/_ref.
#ifndef RPWA_SHIM_MULTI_ARRAY_HPP
#define RPWA_SHIM_MULTI_ARRAY_HPP

#include <algorithm>
#include <array>
#include <cassert>
#include <cstddef>
#include <memory>

#include "boost/array.hpp"

namespace boost {

	namespace detail_shim {

		template<std::size_t N>
		struct extent_gen {
			std::array<std::size_t, N> ranges;
			extent_gen<N + 1> operator[](std::size_t n) const
			{
				extent_gen<N + 1> r;
				std::copy(ranges.begin(), ranges.end(), r.ranges.begin());
				r.ranges[N] = n;
				return r;
			}
		};

		// view of the trailing N dimensions of an array
		template<typename T, std::size_t N>
		struct sub_array {
			T*                 base;
			const std::size_t* shape;    // N extents
			const std::size_t* strides;  // N strides
			typedef sub_array<T, N - 1> next;
			next operator[](std::size_t i) const { return next{base + i * strides[0], shape + 1, strides + 1}; }
		};
		template<typename T>
		struct sub_array<T, 1> {
			T*                 base;
			const std::size_t* shape;
			const std::size_t* strides;
			T& operator[](std::size_t i) const { return base[i]; }
		};

	}  // namespace detail_shim

	static const detail_shim::extent_gen<0> extents = {};

	template<typename T, std::size_t N>
	class multi_array {

	public:

		typedef T           element;
		typedef std::size_t size_type;
		typedef long        index;
		typedef typename std::conditional<(N > 1), detail_shim::sub_array<T, N - 1>, T&>::type reference;
		typedef typename std::conditional<(N > 1), detail_shim::sub_array<const T, N - 1>, const T&>::type const_reference;

		multi_array() { _shape.fill(0); _strides.fill(0); }
		multi_array(const detail_shim::extent_gen<N>& e) { allocate(e.ranges); }
		template<typename I>
		explicit multi_array(const boost::array<I, N>& s)
		{
			std::array<std::size_t, N> sh;
			for (std::size_t d = 0; d < N; ++d)
				sh[d] = (std::size_t)s[d];
			allocate(sh);
		}
		multi_array(const multi_array& o) : _shape(o._shape), _strides(o._strides), _n(o._n)
		{
			_data.reset(new T[_n > 0 ? _n : 1]);
			std::copy(o._data.get(), o._data.get() + _n, _data.get());
		}
		multi_array& operator=(const multi_array& o)
		{
			if (this != &o) {
				multi_array t(o);
				swap(t);
			}
			return *this;
		}

		void resize(const detail_shim::extent_gen<N>& e)
		{
			multi_array t(e);
			// keep the elements whose index lies in both shapes
			std::array<std::size_t, N> lim;
			std::size_t                n = 1;
			for (std::size_t d = 0; d < N; ++d) {
				lim[d] = std::min(_shape[d], t._shape[d]);
				n *= lim[d];
			}
			for (std::size_t k = 0; k < n; ++k) {
				std::size_t r = k, src = 0, dst = 0;
				for (std::size_t d = N; d-- > 0;) {
					const std::size_t i = r % lim[d];
					r /= lim[d];
					src += i * _strides[d];
					dst += i * t._strides[d];
				}
				t._data[dst] = _data[src];
			}
			swap(t);
		}

		reference operator[](std::size_t i) { return at<T>(_data.get(), i); }
		const_reference operator[](std::size_t i) const { return at<const T>(_data.get(), i); }

		T*                 data()               { return _data.get(); }
		const T*           data()         const { return _data.get(); }
		T*                 origin()             { return _data.get(); }
		std::size_t        num_elements() const { return _n; }
		std::size_t        num_dimensions() const { return N; }
		const std::size_t* shape()        const { return _shape.data(); }
		std::size_t        size()         const { return _shape[0]; }

	private:

		template<typename U>
		typename std::enable_if<(N > 1), detail_shim::sub_array<U, N - 1> >::type
		at(U* base, std::size_t i) const
		{
			return detail_shim::sub_array<U, N - 1>{base + i * _strides[0], _shape.data() + 1, _strides.data() + 1};
		}
		template<typename U>
		typename std::enable_if<(N == 1), U&>::type
		at(U* base, std::size_t i) const { return base[i]; }

		void allocate(const std::array<std::size_t, N>& sh)
		{
			_shape = sh;
			_n     = 1;
			for (std::size_t d = N; d-- > 0;) {
				_strides[d] = _n;
				_n *= _shape[d];
			}
			_data.reset(new T[_n > 0 ? _n : 1]());
		}
		void swap(multi_array& o)
		{
			std::swap(_shape, o._shape);
			std::swap(_strides, o._strides);
			std::swap(_n, o._n);
			std::swap(_data, o._data);
		}

		std::array<std::size_t, N> _shape;
		std::array<std::size_t, N> _strides;
		std::size_t                _n = 0;
		std::unique_ptr<T[]>       _data = std::unique_ptr<T[]>(new T[1]());
	};

}  // namespace boost

#endif

// Test-infrastructure shim: the part of the Boost.Accumulators framework that
// the reference's utilities/sumAccumulators.hpp builds on (accumulator_base,
// the `sample` keyword with defaults, depends_on, extractor, as_feature /
// feature_of, stats<> and accumulator_set).  An accumulator_set<T,
// stats<tag::sum(compensated)>> resolves, through the reference's own
// as_feature specialisation, to the reference's compensatedSumAccumulator<T>,
// so the Kahan arithmetic that runs is the reference's, not this file's.
// Only used to compile the reference's own sources into the checker library
// under oracle/_ref.
#ifndef RPWA_SHIM_ACCUMULATORS_HPP
#define RPWA_SHIM_ACCUMULATORS_HPP

namespace boost {

	namespace mpl {
		struct _1 {};
	}

	namespace accumulators {

		struct dont_care {
			template<typename A>
			dont_care(const A&) {}
		};
		struct accumulator_base {};
		template<typename... F>
		struct depends_on {};
		template<typename... F>
		struct stats {};

		namespace tag {
			struct sum {};
			struct sample {};
		}

		template<typename F>
		struct as_feature { typedef F type; };
		template<typename F>
		struct feature_of { typedef F type; };

		// named parameters: `kw | default` and argument packs indexed by keyword
		template<typename Tag, typename D>
		struct kw_default { D value; };
		template<typename Tag>
		struct keyword {
			template<typename D>
			kw_default<Tag, D> operator|(const D& d) const { return kw_default<Tag, D>{d}; }
		};
		static const keyword<tag::sample> sample = {};

		struct no_args {
			template<typename Tag, typename D>
			D operator[](const kw_default<Tag, D>& d) const { return d.value; }
		};
		template<typename T>
		struct sample_args {
			const T& s;
			const T& operator[](const keyword<tag::sample>&) const { return s; }
			template<typename D>
			T operator[](const kw_default<tag::sample, D>&) const { return s; }
			template<typename Tag, typename D>
			D operator[](const kw_default<Tag, D>& d) const { return d.value; }
		};

		template<typename Feature>
		struct extractor {
			template<typename Acc>
			auto operator()(const Acc& a) const -> decltype(a.result()) { return a.result(); }
		};

		namespace detail_shim {
			template<typename Impl, typename T>
			struct bind_placeholder;
			template<template<typename> class TT, typename T>
			struct bind_placeholder<TT<mpl::_1>, T> { typedef TT<T> type; };
			template<typename S>
			struct single_feature;
			template<typename F>
			struct single_feature<stats<F> > { typedef typename as_feature<F>::type type; };
		}

		template<typename T, typename Stats>
		class accumulator_set {
			typedef typename detail_shim::single_feature<Stats>::type                        feature;
			typedef typename detail_shim::bind_placeholder<typename feature::impl, T>::type impl_type;
			impl_type _impl;
		public:
			accumulator_set() : _impl(no_args()) {}
			void operator()(const T& x) { _impl(sample_args<T>{x}); }
			T result() const { return _impl.result(no_args()); }
		};

		template<typename T, typename S>
		T sum(const accumulator_set<T, S>& a) { return a.result(); }

	}  // namespace accumulators

}  // namespace boost

#define BOOST_PARAMETER_NESTED_KEYWORD(tagNamespace, name, alias)          \
	namespace tagNamespace { struct name {}; }                              \
	static const ::boost::accumulators::keyword<tagNamespace::name> name  = {}; \
	static const ::boost::accumulators::keyword<tagNamespace::name> alias = {};
#define BOOST_ACCUMULATORS_IGNORE_GLOBAL(x)

#endif

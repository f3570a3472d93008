// Test-infrastructure shim: the ROOT::Math multi-dimensional function
// interfaces that pwaLikelihood implements (the method set a Minuit2 or
// NLopt driver sees).
#ifndef RPWA_SHIM_IFUNCTION_H
#define RPWA_SHIM_IFUNCTION_H
namespace ROOT {
	namespace Math {
		class IBaseFunctionMultiDim {
		public:
			virtual ~IBaseFunctionMultiDim() {}
			virtual IBaseFunctionMultiDim* Clone() const = 0;
			virtual unsigned int NDim() const = 0;
			double operator()(const double* x) const { return DoEval(x); }
		private:
			virtual double DoEval(const double* x) const = 0;
		};
		class IGradientFunctionMultiDim : public IBaseFunctionMultiDim {
		public:
			virtual IGradientFunctionMultiDim* Clone() const = 0;
			virtual void Gradient(const double* x, double* grad) const = 0;
			virtual void FdF(const double* x, double& f, double* df) const = 0;
			double Derivative(const double* x, unsigned int i) const { return DoDerivative(x, i); }
		private:
			virtual double DoDerivative(const double* x, unsigned int i) const = 0;
		};
	}
}
#endif

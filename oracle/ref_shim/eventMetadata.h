// Test-infrastructure shim: an event file's identity (content hash), its
// event tree and the names of its additional (binning) variables, plus the
// helper that reads those variables per entry and applies an on-the-fly
// bin (a rejection test x < lower or x >= upper, like the reference's
// storageFormats/eventMetadata.cc:380-399).
#ifndef RPWA_SHIM_EVENTMETADATA_H
#define RPWA_SHIM_EVENTMETADATA_H
#include <map>
#include <string>
#include <vector>
#include "TObject.h"
#include "TTree.h"
#include "multibinTypes.h"
namespace rpwa {
	class eventMetadata : public TObject {
	public:
		eventMetadata(const std::string& hash = "", TTree* tree = nullptr,
		              const std::vector<std::string>& vars = std::vector<std::string>())
			: _contentHash(hash), _tree(tree), _vars(vars) {}
		const std::string&              contentHash()                 const { return _contentHash; }
		TTree*                          eventTree()                   const { return _tree; }
		const std::vector<std::string>& additionalTreeVariableNames() const { return _vars; }
	private:
		std::string              _contentHash;
		TTree*                   _tree;
		std::vector<std::string> _vars;
	};
	class additionalTreeVariables {
	public:
		additionalTreeVariables() {}
		additionalTreeVariables(const additionalTreeVariables&) = delete;
		additionalTreeVariables& operator=(const additionalTreeVariables&) = delete;
		double operator[](const std::string& label) const { return _values.at(label); }
		bool setBranchAddresses(const eventMetadata& meta)
		{
			TTree* t = meta.eventTree();
			if (!t)
				return false;
			for (const auto& name : meta.additionalTreeVariableNames())
				if (t->SetBranchAddress(name.c_str(), &_values[name]) < 0) {
					_values.clear();
					return false;
				}
			return true;
		}
		bool inBoundaries(const multibinBoundariesType& bounds) const
		{
			for (const auto& b : bounds) {
				const auto it = _values.find(b.first);
				if (it == _values.end())
					return false;
				if (it->second < b.second.first or it->second >= b.second.second)
					return false;
			}
			return true;
		}
	private:
		std::map<std::string, double> _values;
	};
}
#endif

// Test-infrastructure shim: one wave's amplitude tree with its wave name
// (objectBaseName) and the metadata of the event files it was computed from.
#ifndef RPWA_SHIM_AMPLITUDEMETADATA_H
#define RPWA_SHIM_AMPLITUDEMETADATA_H
#include <string>
#include <vector>
#include "TObject.h"
#include "TTree.h"
#include "eventMetadata.h"
namespace rpwa {
	class amplitudeMetadata : public TObject {
	public:
		amplitudeMetadata(const std::string& name, TTree* tree,
		                  const std::vector<rpwa::eventMetadata>& evtMetas = std::vector<rpwa::eventMetadata>())
			: _name(name), _tree(tree), _evtMetas(evtMetas) {}
		const std::vector<rpwa::eventMetadata>& eventMetadata()  const { return _evtMetas; }
		const std::string&                      objectBaseName() const { return _name; }
		TTree*                                  amplitudeTree()  const { return _tree; }
		static inline const std::string amplitudeLeafName = "amplitude";
	private:
		std::string                      _name;
		TTree*                           _tree;
		std::vector<rpwa::eventMetadata> _evtMetas;
	};
}
#endif

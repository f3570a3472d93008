// Test-infrastructure shim: a wave description reduced to what the
// likelihood reads from it (the reflectivity of X, through the decay
// topology's X vertex), so that pwaLikelihood::readWaveList runs unchanged.
#ifndef RPWA_SHIM_WAVEDESCRIPTION_H
#define RPWA_SHIM_WAVEDESCRIPTION_H
#include <memory>
#include "TObject.h"
namespace rpwa {
	class amplitudeMetadata;  // declared through the key-file headers in the reference
	class particle {
	public:
		explicit particle(int refl) : _refl(refl) {}
		int reflectivity() const { return _refl; }
	private:
		int _refl;
	};
	typedef std::shared_ptr<particle> particlePtr;
	class isobarDecayVertex {
	public:
		explicit isobarDecayVertex(particlePtr p) : _parent(p) {}
		const particlePtr& parent() const { return _parent; }
	private:
		particlePtr _parent;
	};
	typedef std::shared_ptr<isobarDecayVertex> isobarDecayVertexPtr;
	class isobarDecayTopology {
	public:
		explicit isobarDecayTopology(int refl) : _x(new isobarDecayVertex(particlePtr(new particle(refl)))) {}
		const isobarDecayVertexPtr& XIsobarDecayVertex() const { return _x; }
	private:
		isobarDecayVertexPtr _x;
	};
	typedef std::shared_ptr<isobarDecayTopology> isobarDecayTopologyPtr;
	class waveDescription : public TObject {
	public:
		explicit waveDescription(int reflectivity = +1) : _refl(reflectivity) {}
		bool constructDecayTopology(isobarDecayTopologyPtr& topo, const bool = false) const
		{
			topo.reset(new isobarDecayTopology(_refl));
			return true;
		}
		bool keyFileParsed() const { return false; }
	private:
		int _refl;
	};
}
#endif

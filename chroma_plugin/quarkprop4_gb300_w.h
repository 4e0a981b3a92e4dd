// -*- C++ -*-
/*! \file
 *  \brief Batched propagator solve for GB300_CLOVER_INVERTER: the counterpart of quarkProp4_a.
 *
 *  Chroma's quarkProp4_a (lib/actions/ferm/qprop/quarkprop4_w.cc:31-175), reached from
 *  WilsonTypeFermAct::quarkProp (:270-275), calls the factory solver once per spin-colour source.
 *  Through the factory entry alone the GB300 library therefore sees 12 single-right-hand-side
 *  even-odd solves, each after Chroma's host-side Schur preparation (PrecFermActQprop,
 *  eoprec_fermact_qprop.cc:41-80).  A propagator caller whose invParam names
 *  GB300_CLOVER_INVERTER can call quarkProp4GB300 in place of S_f->quarkProp(...): it extracts
 *  the sources like quarkProp4_a (PropToFerm, each normalised to |chi| = 1), solves all of them as
 *  one multi-right-hand-side batch of the full system on the device (Schur preparation, odd solve
 *  and even reconstruction included, GBC_SYS_FULL), undoes the normalisation and fills q_sol
 *  (FermToProp), with the same per-source Qprop records in xml_out and the same
 *  QUARK_SPIN_TYPE_UPPER / _LOWER handling (half the sources solved, the other columns the
 *  gamma_5-negated copies).
 *  Compiled only inside a Chroma build (needs QDP++).
 */
#ifndef __quarkprop4_gb300_w_h__
#define __quarkprop4_gb300_w_h__

#include "chromabase.h"
#include "handle.h"
#include "state.h"
#include "io/enum_io/enum_quarkspintype_io.h"
#include "io/xml_group_reader.h"

namespace Chroma
{
  void quarkProp4GB300(LatticePropagator& q_sol, XMLWriter& xml_out, const LatticePropagator& q_src,
                       Handle<FermState<LatticeFermion, multi1d<LatticeColorMatrix>, multi1d<LatticeColorMatrix> > > state,
                       const GroupXML_t& invParam, QuarkSpinType quarkSpinType, int& ncg_had);
}  // namespace Chroma

#endif

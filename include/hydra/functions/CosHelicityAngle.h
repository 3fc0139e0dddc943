// CosHelicityAngle.h -- cosine of the helicity angle of daughter D of Q, itself a daughter of P,
// as the reference's hydra::CosHelicityAngle (hydra/functions/CosHelicityAngle.h) computes it from
// Minkowski products: (P.D mQ^2 - P.Q Q.D) / sqrt(((P.Q)^2 - mQ^2 mP^2) ((Q.D)^2 - mQ^2 mD^2)).
// Callable in host and device code; usable inside a wrap_lambda functor.
#pragma once
#include "../hps_phasespace.hpp"

namespace hydra {

class CosHelicityAngle {
public:
    CosHelicityAngle() = default;
    HPS_HD double operator()(Vector4R const& P, Vector4R const& Q, Vector4R const& D) const
    {
        const double pd = P * D, pq = P * Q, qd = Q * D;
        const double mp2 = P.mass2(), mq2 = Q.mass2(), md2 = D.mass2();
        return (pd * mq2 - pq * qd) / ::sqrt((pq * pq - mq2 * mp2) * (qd * qd - mq2 * md2));
    }
};

}  // namespace hydra

"""
The ChainRulesCore `rrule` of `PTDiffusion.misfit`: the forward solve with one
checkpoint per physical step, and a pullback that runs the library's adjoint
(`ptd_adj_gradient`) for the gradients with respect to m and H0.  A package
extension, so the rule exists whenever PTDiffusion and ChainRulesCore are both
loaded, whatever the load order.
"""
module PTDiffusionChainRulesCoreExt

using PTDiffusion: PTDiffusion, AdjointSolver, forward!, gradient!, misfit
import ChainRulesCore

function ChainRulesCore.rrule(::typeof(misfit), a::AdjointSolver, m, H0, Ht)
    L = forward!(a, H0, m, Ht)
    function misfit_pullback(dL)
        gm, gh = gradient!(a)
        return ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), dL .* gm, dL .* gh,
               ChainRulesCore.NoTangent()
    end
    return L, misfit_pullback
end

end # module

# ChainRulesCore rule of the GPU density loss: a package extension, loaded only when the user
# also loads ChainRulesCore (directly or through Zygote and the like), so the glue itself does
# not depend on it.
module LatticeModelsGB300ChainRulesCoreExt

using LatticeModelsGB300: DensityLossProblem, density_loss, loss_and_gradients
import ChainRulesCore

# One forward pass with checkpoints and the hand-written adjoint give the loss and both
# gradients; the pullback only scales them.
function ChainRulesCore.rrule(::typeof(density_loss), V, B, p::DensityLossProblem)
    loss, gV, gB = loss_and_gradients(p, Vector{Float64}(V), Vector{Float64}(B))
    pullback(dl) = (ChainRulesCore.NoTangent(), dl .* gV, dl .* gB, ChainRulesCore.NoTangent())
    return loss, pullback
end

end # module

"""The CUDA substrate: drop-in counterpart of ``gigalens.tf`` on GB300.

    gigalens.tf.profiles.mass.epl.EPL          -> gigalens_gb300.cuda.profiles.mass.epl.EPL
    gigalens.tf.profiles.light.sersic.*        -> gigalens_gb300.cuda.profiles.light.sersic.*
    gigalens.tf.simulator.LensSimulator        -> gigalens_gb300.cuda.simulator.LensSimulator
    gigalens.tf.model.ForwardProbModel         -> gigalens_gb300.cuda.model.ForwardProbModel
    gigalens.tf.inference.ModellingSequence    -> gigalens_gb300.cuda.inference.ModellingSequence
"""

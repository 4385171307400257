/* Generated by crtrig_tables.py (400-bit mpmath); do not edit. */
#ifndef LIFE_CRTRIG_TABLES_H
#define LIFE_CRTRIG_TABLES_H

/* atan(k/256), k = 0..256: hi, lo pairs */
#define LIFE_CR_ATAN256 \
    0.0, 0.0, \
    0x1.ffff5555bbbb7p-9, 0x1.4bb12afb6b6d5p-64, \
    0x1.fffd555bbba97p-8, 0x1.68062351fbbe6p-63, \
    0x1.7ffb80184c30ap-7, -0x1.725017508234bp-61, \
    0x1.fff555bbb729bp-7, -0x1.220c39d4dff50p-61, \
    0x1.3ff595f18a700p-6, -0x1.213eac36cfb2cp-60, \
    0x1.7fee0184a5c36p-6, -0x1.43189fc0a354bp-60, \
    0x1.bfe36df291712p-6, -0x1.e1bec7756100ep-61, \
    0x1.ffd55bba97625p-6, -0x1.5ec431444912cp-60, \
    0x1.1fe1a5c2ec497p-5, 0x1.886091e8fc4cbp-59, \
    0x1.3fd65f169c9d9p-5, 0x1.7230a716461b5p-61, \
    0x1.5fc89a5fa3b2dp-5, 0x1.2bb73bf4e7f99p-59, \
    0x1.7fb818430da2ap-5, -0x1.86ef8f794f105p-63, \
    0x1.9fa49986984dfp-5, 0x1.322907af0abc2p-59, \
    0x1.bf8ddf139c444p-5, -0x1.89fe34b2a7fa8p-59, \
    0x1.df73a9f9f1882p-5, -0x1.251b5c410bcb4p-62, \
    0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60, \
    0x1.0f99ea71d52a7p-4, -0x1.2069feec3624fp-61, \
    0x1.1f86dbf082d59p-4, -0x1.095dc7732ef81p-59, \
    0x1.2f719318a4a9ap-4, 0x1.3fd1779b9801fp-63, \
    0x1.3f59f0e7c559dp-4, 0x1.ac4ce285df847p-58, \
    0x1.4f3fd677292fbp-4, 0x1.008d36264979ep-59, \
    0x1.5f2324fd2d7b2p-4, 0x1.8a8da4401318ep-58, \
    0x1.6f03bdcea4b0dp-4, -0x1.3f00e512fa17dp-60, \
    0x1.7ee182602f10fp-4, -0x1.cfb654c0c3d98p-58, \
    0x1.8ebc54478fb28p-4, 0x1.732880cad24ccp-59, \
    0x1.9e94153cfdcf1p-4, 0x1.a332e1d69c47ep-58, \
    0x1.ae68a71c722b8p-4, 0x1.c014e6910b9dbp-59, \
    0x1.be39ebe6f07c3p-4, 0x1.f7b8f29a05987p-58, \
    0x1.ce07c5c3cca32p-4, 0x1.138e6425918a7p-59, \
    0x1.ddd21701eba6ep-4, 0x1.94effcd76fe58p-58, \
    0x1.ed98c2190043bp-4, -0x1.3a598592c7b13p-61, \
    0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59, \
    0x1.068d584212b3ep-3, -0x1.9e2d283019bfdp-57, \
    0x1.0e6adccf40882p-3, -0x1.d71a31bb98d0dp-57, \
    0x1.1646541060850p-3, 0x1.6bcee8ae7ea92p-57, \
    0x1.1e1fafb043727p-3, -0x1.b485914dacf8cp-59, \
    0x1.25f6e171a535cp-3, 0x1.7c6d7bde1a310p-57, \
    0x1.2dcbdb2fba1ffp-3, 0x1.8f28705561534p-58, \
    0x1.359e8edeb99a4p-3, -0x1.a5fd74e4604c6p-57, \
    0x1.3d6eee8c6626cp-3, 0x1.61a3b0ce9281bp-57, \
    0x1.453cec6092a9ep-3, 0x1.1f653b3a5a78bp-57, \
    0x1.4d087a9da4f17p-3, 0x1.1f323f1adf158p-57, \
    0x1.54d18ba11570ap-3, 0x1.18282f2884073p-57, \
    0x1.5c9811e3ec26ap-3, -0x1.054ab2c010f3dp-58, \
    0x1.645bfffb3aa74p-3, -0x1.f536b677c2cb4p-60, \
    0x1.6c1d4898933d9p-3, -0x1.2954a7603c427p-58, \
    0x1.73dbde8a7d202p-3, -0x1.5ad0f6d4a665dp-58, \
    0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58, \
    0x1.8350be398ebc8p-3, -0x1.5a91332b9c90dp-58, \
    0x1.8b06ee2879c29p-3, -0x1.118cd30308c4fp-57, \
    0x1.92ba37d050272p-3, -0x1.0d3ded0ff4764p-57, \
    0x1.9a6a8e96c8626p-3, 0x1.cf601e7b4348ep-59, \
    0x1.a217e601081a6p-3, -0x1.0def8a60af374p-57, \
    0x1.a9c231b403279p-3, 0x1.0e8bbe89cca85p-57, \
    0x1.b1696574d780cp-3, -0x1.85ab8fc15a673p-58, \
    0x1.b90d7529260a2p-3, 0x1.17b10d2e0e5abp-61, \
    0x1.c0ae54d768467p-3, -0x1.04cdbf55f26dcp-57, \
    0x1.c84bf8a742e6ep-3, -0x1.95bdd0682ea26p-58, \
    0x1.cfe654e1d5395p-3, 0x1.47b9a3f71eafbp-57, \
    0x1.d77d5df205736p-3, 0x1.c648d1534597ep-57, \
    0x1.df110864c9d9ep-3, -0x1.5818b53bf4781p-60, \
    0x1.e6a148e96ec4dp-3, 0x1.866b22029f765p-57, \
    0x1.ee2e1451d980dp-3, -0x1.9a7708c46ba91p-58, \
    0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57, \
    0x1.fd3d1fc40dbe4p-3, 0x1.37146f3a1c5eap-59, \
    0x1.025fa510665b6p-2, -0x1.672df6832fa48p-56, \
    0x1.061eea03d6291p-2, -0x1.5f760db154301p-59, \
    0x1.09dc597d86362p-2, 0x1.62e47390cb865p-56, \
    0x1.0d97ee509acb3p-2, 0x1.47c317bd5a3ebp-56, \
    0x1.1151a362431cap-2, -0x1.4dc8dc9077b9fp-56, \
    0x1.150973a9ce547p-2, -0x1.796ba7f9ca328p-56, \
    0x1.18bf5a30bf178p-2, 0x1.30ca4748b1bf9p-57, \
    0x1.1c735212dd884p-2, -0x1.7d9ac78cb2f2ep-57, \
    0x1.2025567e47c96p-2, -0x1.1832328f4290ep-57, \
    0x1.23d562b381042p-2, -0x1.c531716200088p-58, \
    0x1.278372057ef46p-2, -0x1.077cdd36dfc81p-56, \
    0x1.2b2f7fd9b5fe2p-2, 0x1.423cfc1c2d443p-61, \
    0x1.2ed987a823cfep-2, 0x1.b91258ea012cap-57, \
    0x1.328184fb58952p-2, -0x1.a95f0a9939f2fp-56, \
    0x1.362773707ebccp-2, -0x1.963a544b672d8p-57, \
    0x1.39cb4eb76157cp-2, -0x1.2f4da5a214713p-56, \
    0x1.3d6d129271134p-2, 0x1.137ca41cc958ap-56, \
    0x1.410cbad6c7d33p-2, -0x1.b0c8bae13b512p-56, \
    0x1.44aa436c2af0ap-2, -0x1.5d5e43c55b3bap-56, \
    0x1.4845a84d0c21bp-2, 0x1.1e28a7563c6a6p-56, \
    0x1.4bdee586890e7p-2, -0x1.e4dc77c22a757p-57, \
    0x1.4f75f73869979p-2, -0x1.95a1cf7ff1108p-58, \
    0x1.530ad9951cd4ap-2, -0x1.2566480884082p-57, \
    0x1.569d88e1b4cd8p-2, -0x1.fec61e713cfe2p-57, \
    0x1.5a2e0175e0f4ep-2, 0x1.13b7a8f82e457p-56, \
    0x1.5dbc3fbbe768dp-2, 0x1.ea0ec1b76f7dap-57, \
    0x1.614840309cfe2p-2, -0x1.a725715711f00p-56, \
    0x1.64d1ff635c1c6p-2, -0x1.fa403e7c0fdbep-56, \
    0x1.685979f5fa6fep-2, -0x1.257814d1ada9cp-59, \
    0x1.6bdeac9cbd76dp-2, -0x1.a5c563e6de828p-58, \
    0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56, \
    0x1.72e22d53aa2aap-2, -0x1.d9c934e79f27cp-56, \
    0x1.7660752817502p-2, -0x1.dd11791cc7600p-59, \
    0x1.79dc6899118d1p-2, 0x1.b7413a0ef606dp-61, \
    0x1.7d5604b63b3f7p-2, 0x1.69c885c2b249ap-56, \
    0x1.80cd46a14b1d1p-2, -0x1.e79f99684fa19p-56, \
    0x1.84422b8df95d7p-2, 0x1.d76a0299b41b6p-56, \
    0x1.87b4b0c1ebedcp-2, -0x1.6dcfaa2fa470fp-56, \
    0x1.8b24d394a1b25p-2, 0x1.b6d0ba3748fa8p-56, \
    0x1.8e92916f5cde8p-2, 0x1.4c0a7e12bfafbp-56, \
    0x1.91fde7cd0c662p-2, 0x1.1074188054b53p-56, \
    0x1.9566d43a34907p-2, 0x1.9b01537e0af2bp-57, \
    0x1.98cd5454d6b18p-2, 0x1.9e6c988fd0a77p-56, \
    0x1.9c3165cc58107p-2, 0x1.b669602250cfbp-59, \
    0x1.9f93066168002p-2, -0x1.c827047c9439ap-56, \
    0x1.a2f233e5e530bp-2, 0x1.814d5f797086bp-58, \
    0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56, \
    0x1.a9a92d59e98cfp-2, 0x1.2e42dff75d817p-59, \
    0x1.ad00f5422058bp-2, 0x1.fc4c33891d2e8p-56, \
    0x1.b056420ae9344p-2, -0x1.9313946363455p-56, \
    0x1.b3a911da65c6cp-2, 0x1.ae187b1ca5040p-56, \
    0x1.b6f962e737efcp-2, -0x1.ca53464981e71p-58, \
    0x1.ba473378624a5p-2, 0x1.519a1b46e4affp-56, \
    0x1.bd9281e528192p-2, -0x1.4b15439af6b66p-56, \
    0x1.c0db4c94ec9f0p-2, -0x1.cc1ce70934c34p-56, \
    0x1.c42191ff11eb7p-2, -0x1.b17df434b3eeep-56, \
    0x1.c76550aad71f9p-2, -0x1.74b8bff7043e4p-56, \
    0x1.caa6872f3631bp-2, 0x1.9506781636f48p-61, \
    0x1.cde53432c1351p-2, -0x1.a2cfa4418f1adp-56, \
    0x1.d121566b7f2adp-2, 0x1.be67835886c30p-56, \
    0x1.d45aec9ec862bp-2, 0x1.89421163ef92dp-57, \
    0x1.d791f5a1226f5p-2, -0x1.4017ea5b64a76p-57, \
    0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56, \
    0x1.ddf85bb026974p-2, 0x1.43bbb0c0a1226p-57, \
    0x1.e127b6b0744b0p-2, -0x1.2b0986398d4abp-58, \
    0x1.e4548066cf51ap-2, 0x1.3a3aa12ce98f2p-59, \
    0x1.e77eb7f175a34p-2, 0x1.0e53dc1bf3435p-56, \
    0x1.eaa65c7cf28c4p-2, 0x1.2fb2ceca3bf05p-57, \
    0x1.edcb6d43f8435p-2, -0x1.fc976330884e4p-58, \
    0x1.f0ede98f393d0p-2, -0x1.2f40a87cb1894p-56, \
    0x1.f40dd0b541418p-2, -0x1.a3992dc382a23p-57, \
    0x1.f72b221a4e495p-2, 0x1.489c20f7eb740p-58, \
    0x1.fa45dd3029259p-2, -0x1.ca563dc28d8b5p-56, \
    0x1.fd5e0175fdf83p-2, 0x1.3a87b1ec49b15p-57, \
    0x1.0039c73c1a40cp-1, -0x1.b32c949c9d593p-55, \
    0x1.01c341e82422dp-1, 0x1.3db44fcca90eep-55, \
    0x1.034b709250488p-1, 0x1.8f9b38d855410p-56, \
    0x1.04d25314342e6p-1, -0x1.1c8636442c767p-55, \
    0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56, \
    0x1.07dc3324e9b38p-1, 0x1.b70c9e04450acp-56, \
    0x1.095f30861a590p-1, -0x1.121b20a15a9f3p-56, \
    0x1.0ae0e1639866cp-1, 0x1.075abf2de445ap-56, \
    0x1.0c6145b5b43dap-1, 0x1.974fa13b5404fp-58, \
    0x1.0de05d7aa6f7dp-1, -0x1.83684b1c529abp-56, \
    0x1.0f5e28b67e295p-1, 0x1.311b17ec990d0p-65, \
    0x1.10daa77307a0dp-1, 0x1.69c33d44c7b05p-55, \
    0x1.1255d9bfbd2a9p-1, -0x1.2bdaee1c0ee35p-58, \
    0x1.13cfbfb1b056ep-1, 0x1.3110e6fc3ed38p-55, \
    0x1.154859637646ap-1, -0x1.4ba7c548bf3c3p-55, \
    0x1.16bfa6f5137e1p-1, 0x1.9606fe141bd35p-56, \
    0x1.1835a88be7c13p-1, 0x1.c621cec00c301p-55, \
    0x1.19aa5e5299f9ap-1, -0x1.a606c2c58f835p-55, \
    0x1.1b1dc87904285p-1, -0x1.21e8c8aef8f29p-57, \
    0x1.1c8fe7341f64fp-1, 0x1.28bbc9d5e792ap-56, \
    0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58, \
    0x1.1f7043557138ap-1, 0x1.6c659f6d7dd47p-56, \
    0x1.20de813e823b2p-1, -0x1.791d753ebb744p-55, \
    0x1.224b74c1d192ap-1, 0x1.d6d3df88a60c4p-55, \
    0x1.23b71e2cc9e6ap-1, 0x1.c421c9f38224ep-57, \
    0x1.25217dd17e501p-1, 0x1.56aa88c1b679cp-55, \
    0x1.268a940696da6p-1, 0x1.d1348a04c73ccp-58, \
    0x1.27f261273d1b3p-1, 0x1.43bf36151dd9fp-55, \
    0x1.2958e59308e31p-1, -0x1.09e73b0c6c087p-56, \
    0x1.2abe21aded073p-1, 0x1.c28c001ad022ep-55, \
    0x1.2c2215e024466p-1, -0x1.4b810da3a4be1p-59, \
    0x1.2d84c2961e48cp-1, -0x1.f25420a36e506p-56, \
    0x1.2ee628406cbcap-1, 0x1.c5d5e9ff0cf8dp-55, \
    0x1.30464753b090bp-1, -0x1.3e71261da18f3p-56, \
    0x1.31a52048874bep-1, 0x1.40cab87a7ac24p-55, \
    0x1.3302b39b78856p-1, 0x1.5dd2ed87ba82bp-55, \
    0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55, \
    0x1.35ba0b60ecccep-1, 0x1.e3ba19b9368b9p-55, \
    0x1.3713d0df6c504p-1, -0x1.4f789e031606dp-58, \
    0x1.386c52d3db11fp-1, -0x1.b78e1cbebe6a0p-55, \
    0x1.39c391cd4171ap-1, -0x1.2304331d8bf46p-55, \
    0x1.3b198e5e2564bp-1, -0x1.2f9221f0752acp-56, \
    0x1.3c6e491c78dc5p-1, -0x1.e145094fd0ba7p-55, \
    0x1.3dc1c2a188504p-1, 0x1.2ce6370f4e971p-55, \
    0x1.3f13fb89e96f4p-1, 0x1.ecf8b492644f0p-56, \
    0x1.4064f47569f49p-1, -0x1.aad88f91bf2b2p-55, \
    0x1.41b4ae06fea41p-1, 0x1.3d60a53277652p-57, \
    0x1.430328e4b26d6p-1, -0x1.131591070b99fp-55, \
    0x1.445065b795b56p-1, -0x1.f76d0163f79c8p-56, \
    0x1.459c652badc7fp-1, 0x1.199698e8e135cp-55, \
    0x1.46e727efe4716p-1, -0x1.39b9b1b844cc9p-57, \
    0x1.4830aeb5f7bfep-1, -0x1.a265666764a73p-58, \
    0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56, \
    0x1.4ac00b1c71762p-1, 0x1.b20e72382b900p-55, \
    0x1.4c05e22de94e5p-1, -0x1.c0ac1f09f2edfp-55, \
    0x1.4d4a8023414e8p-1, 0x1.e3a891daa88b0p-57, \
    0x1.4e8de5bb6ec04p-1, 0x1.4a33dbeb3796cp-55, \
    0x1.4fd013b7dd17ep-1, 0x1.d513f3e7c24b5p-56, \
    0x1.51110adc5ed81p-1, 0x1.23dcd6832a63ep-56, \
    0x1.5250cbef1e9fbp-1, -0x1.539b7a3228870p-58, \
    0x1.538f57b89061fp-1, -0x1.1bb74abda520cp-55, \
    0x1.54ccaf0362c8fp-1, 0x1.8a3247f8f43c1p-55, \
    0x1.5608d29c70c34p-1, 0x1.9939cf0de8088p-55, \
    0x1.5743c352b33bap-1, -0x1.ea00d34c87ea6p-55, \
    0x1.587d81f732fbbp-1, -0x1.5e5c9d8c5a950p-56, \
    0x1.59b60f5cfab9ep-1, -0x1.1b04c41026bc5p-55, \
    0x1.5aed6c5909517p-1, 0x1.7312f714a9436p-55, \
    0x1.5c2399c244261p-1, -0x1.31bd4e9e56b35p-55, \
    0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57, \
    0x1.5e8c6941043d0p-1, -0x1.0bf75be451e70p-56, \
    0x1.5fbf0d0d5cc4ap-1, -0x1.b4cfd000b7158p-58, \
    0x1.60f084b46e05fp-1, -0x1.dbb8699945193p-55, \
    0x1.6220d115d7b8ep-1, -0x1.2b785350ee8c1p-57, \
    0x1.634ff312d1f3bp-1, 0x1.9d2f315f2b598p-55, \
    0x1.647deb8e20b90p-1, -0x1.eca04023a51cfp-58, \
    0x1.65aabb6c07b03p-1, -0x1.7939b3af32729p-57, \
    0x1.66d663923e087p-1, -0x1.6ea6febe8bbbap-56, \
    0x1.6800e4e7e2858p-1, -0x1.8ea6a1b3e90f0p-58, \
    0x1.692a40556fb6ap-1, 0x1.d94b95a8ea2ccp-55, \
    0x1.6a5276c4b0576p-1, -0x1.f6b659c46a69ep-55, \
    0x1.6b798920b3d99p-1, -0x1.a80386188c50ep-55, \
    0x1.6c9f7855c3198p-1, 0x1.c09de29bd280dp-56, \
    0x1.6dc44551553afp-1, -0x1.bf8863573828ep-58, \
    0x1.6ee7f10204aefp-1, 0x1.692eea3066272p-55, \
    0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56, \
    0x1.712be84295198p-1, 0x1.5cd90337d8881p-55, \
    0x1.724c35b4fae7bp-1, 0x1.948b32db3499bp-58, \
    0x1.736b65a172dffp-1, 0x1.775fd06a892d1p-56, \
    0x1.748978fba8e0fp-1, 0x1.7b2a6165884a1p-59, \
    0x1.75a670b82d8d8p-1, 0x1.ee4ac4c729087p-55, \
    0x1.76c24dcc6c6c0p-1, 0x1.1952551adc83dp-55, \
    0x1.77dd112ea22c7p-1, 0x1.732608fc10d3dp-55, \
    0x1.78f6bbd5d315ep-1, 0x1.406a089803740p-55, \
    0x1.7a0f4eb9c19a2p-1, 0x1.13c67cd815f57p-57, \
    0x1.7b26cad2e50fep-1, -0x1.ce80df30411fbp-55, \
    0x1.7c3d311a6092bp-1, 0x1.bb3cb2d303288p-55, \
    0x1.7d528289fa093p-1, 0x1.560821e2f3aa9p-55, \
    0x1.7e66c01c114fep-1, -0x1.c82b88b760b8dp-55, \
    0x1.7f79eacb97898p-1, 0x1.fd5ca80ead221p-55, \
    0x1.808c03940694bp-1, -0x1.00f327715f6a5p-55, \
    0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56, \
    0x1.82ad036000005p-1, 0x1.4592fce924d24p-56, \
    0x1.83bbec5cdee22p-1, 0x1.3107104ffc6c3p-57, \
    0x1.84c9c7653f7ebp-1, -0x1.83611fe0a3e8fp-60, \
    0x1.85d69576cc2c5p-1, 0x1.6b66e7fc8b8c3p-57, \
    0x1.86e2578f87ae5p-1, 0x1.022b1375cfe34p-55, \
    0x1.87ed0eadc5a2ap-1, 0x1.0af5ad957f4bcp-56, \
    0x1.88f6bbd023119p-1, -0x1.32d1d25aba660p-58, \
    0x1.89ff5ff57f1f8p-1, -0x1.55b9a5e177a1bp-55, \
    0x1.8b06fc1cf3dffp-1, -0x1.0fb312656db6dp-55, \
    0x1.8c0d9145cf49dp-1, 0x1.bea4076dc4333p-55, \
    0x1.8d13206f8c4cbp-1, -0x1.b018cbaa89a8bp-56, \
    0x1.8e17aa99cc05ep-1, -0x1.ec182ab042f61p-56, \
    0x1.8f1b30c44f167p-1, 0x1.dd1cab93933fdp-57, \
    0x1.901db3eeef187p-1, 0x1.68665e5603c8fp-55, \
    0x1.911f35199833bp-1, 0x1.3ae8a0edbf522p-57, \
    0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55,

/* sin(j/128), cos(j/128), j = 0..101: sin hi, sin lo, cos hi, cos lo */
#define LIFE_CR_SINCOS128 \
    0.0, 0.0, 0x1.0000000000000p+0, 0.0, \
    0x1.fffeaaaaeeeefp-8, -0x1.e45e2ec67b77cp-62, 0x1.fffc000155552p-1, 0x1.f4a01a0196daep-55, \
    0x1.fffaaaaeeeed5p-7, -0x1.2ab639a9f0776p-63, 0x1.fff000155549fp-1, 0x1.28a28a03a5ef3p-55, \
    0x1.7ff7001033255p-6, 0x1.efe2b51527336p-64, 0x1.ffdc006bff7e6p-1, 0x1.ae6dae86977bdp-55, \
    0x1.ffeaaaeeee86fp-6, -0x1.cd406fb224ae2p-60, 0x1.ffc00155527d3p-1, -0x1.3b54492d89b5bp-55, \
    0x1.3feb2b12d45d5p-5, 0x1.4ec54203d1c11p-60, 0x1.ff9c03414a7bap-1, 0x1.991f4be6c59bfp-57, \
    0x1.7fdc01032fba9p-5, -0x1.599bdf46e997ap-59, 0x1.ff7006bfdf99fp-1, -0x1.8b3b560648d5fp-56, \
    0x1.bfc6d78586dacp-5, 0x1.8e4fd03dbf236p-62, 0x1.ff3c0c8103a31p-1, 0x1.4856dbddc0e66p-56, \
    0x1.ffaaaeeed4edbp-5, -0x1.2d16d32684b69p-59, 0x1.ff0015549f4d3p-1, 0x1.328387b99426fp-55, \
    0x1.1fc343d808befp-4, -0x1.f3d32e6f3be4fp-58, 0x1.febc222a8ef9fp-1, 0x1.7934934f54c77p-58, \
    0x1.3facb12d1755bp-4, -0x1.921915299468bp-58, 0x1.fe7034129ef6fp-1, -0x1.cbf4337c96f97p-57, \
    0x1.5f911fd10b737p-4, -0x1.0184f02be9102p-58, 0x1.fe1c4c3c873ebp-1, -0x1.5a9c9057c4a02p-60, \
    0x1.7f701032550e4p-4, 0x1.afc2d1800501ap-60, 0x1.fdc06bf7e6b9bp-1, 0x1.31902b535f8dbp-55, \
    0x1.9f4902d55d1f9p-4, 0x1.2696d7eac1dc1p-58, 0x1.fd5c94b43e000p-1, -0x1.2e768cb4f92f9p-57, \
    0x1.bf1b78568391dp-4, 0x1.e91841dea4cc8p-58, 0x1.fcf0c800e99b1p-1, 0x1.ea3d786d186acp-57, \
    0x1.dee6f16c1cce6p-4, -0x1.50f8e2fb71673p-59, 0x1.fc7d078d1bc88p-1, 0x1.075d2447db685p-55, \
    0x1.feaaeee86ee36p-4, -0x1.afcb2bcc6f03bp-59, 0x1.fc015527d5bd3p-1, 0x1.b68f35094efb8p-55, \
    0x1.0f3378ddd71d1p-3, 0x1.d8468724f0f9ep-57, 0x1.fb7db2bfe0695p-1, 0x1.21dadf4f65ab1p-55, \
    0x1.1f0d3d7afceafp-3, -0x1.6ef95099769a5p-57, 0x1.faf22263c4bd3p-1, -0x1.52ace133a2769p-58, \
    0x1.2ee285e4ab88fp-3, -0x1.e4d0f05dee058p-57, 0x1.fa5ea641c36f2p-1, 0x1.04da6ed17cc7cp-59, \
    0x1.3eb312c5d66cbp-3, 0x1.47d666b66cb91p-57, 0x1.f9c340a7cc428p-1, 0x1.c5b6b063b7462p-55, \
    0x1.4e7ea4dc5f27bp-3, 0x1.949db2ac072fcp-58, 0x1.f91ff40374d01p-1, -0x1.7d03f4d3a9e4cp-57, \
    0x1.5e44fcfa126f3p-3, -0x1.6f443063f89b6p-57, 0x1.f874c2e1eecf6p-1, -0x1.c6514e1332b16p-55, \
    0x1.6e05dc05a4d4cp-3, -0x1.32c5c8b81c919p-66, 0x1.f7c1afeffde24p-1, -0x1.8f55bc47540b1p-56, \
    0x1.7dc102fbaf2b5p-3, 0x1.5ab50e23c97c3p-59, 0x1.f706bdf9ece1cp-1, -0x1.698c80c36dcb4p-55, \
    0x1.8d7632efaa944p-3, -0x1.20fa262cbb953p-57, 0x1.f643efeb82acdp-1, 0x1.6b00ac1fe28acp-56, \
    0x1.9d252d0cec312p-3, 0x1.9c43d80b1137dp-58, 0x1.f57948cff6797p-1, 0x1.e3a0d3e03b1d4p-57, \
    0x1.accdb297a0765p-3, -0x1.9883b57d6cdeap-58, 0x1.f4a6cbd1e3a79p-1, 0x1.13df0edaebb57p-55, \
    0x1.bc6f84edc6199p-3, 0x1.9c1a56a7b0cabp-57, 0x1.f3cc7c3b3d16ep-1, -0x1.21a3ad28a3494p-57, \
    0x1.cc0a6588289a3p-3, -0x1.868d09bc87c6bp-57, 0x1.f2ea5d753ffedp-1, 0x1.cc4215f56d583p-55, \
    0x1.db9e15fb5a5d0p-3, -0x1.32e20d6cc6fc2p-57, 0x1.f20073086649fp-1, 0x1.b940416c1984bp-56, \
    0x1.eb2a57f8ae5a3p-3, -0x1.0be06af572cebp-57, 0x1.f10ec09c5873bp-1, 0x1.d9072762c1283p-55, \
    0x1.faaeed4f31577p-3, -0x1.15d88508e32b8p-57, 0x1.f01549f7deea1p-1, 0x1.d3c1e99e5cafdp-55, \
    0x1.0515cbf65155cp-2, -0x1.9b8c29dfd8ec7p-56, 0x1.ef141300d2f26p-1, -0x1.2aa1b08ded372p-55, \
    0x1.0cd00cef36436p-2, -0x1.9fb0a0c93e2b4p-56, 0x1.ee0b1fbc0f11cp-1, -0x1.bfd2380bbc3b1p-59, \
    0x1.14861aa94ddebp-2, -0x1.be881b5b615a4p-57, 0x1.ecfa744d5efa1p-1, -0x1.56d0a4af541d0p-58, \
    0x1.1c37d64c6b876p-2, 0x1.46076fe0dcff4p-56, 0x1.ebe214f76efa8p-1, -0x1.02f9f12ba543ep-55, \
    0x1.23e52111aaf36p-2, -0x1.4f080334eff18p-56, 0x1.eac2061bbaf4fp-1, 0x1.2c1d53e94658dp-57, \
    0x1.2b8ddc43eb49fp-2, 0x1.1553899f2d807p-57, 0x1.e99a4c3a7cd83p-1, -0x1.2264b1bc53ce8p-55, \
    0x1.3331e94049f87p-2, 0x1.e0cb6b40c302cp-56, 0x1.e86aebf29a9edp-1, 0x1.9397afdbb58a7p-55, \
    0x1.3ad129769d3d8p-2, 0x1.03d550487839ap-63, 0x1.e733ea0193d40p-1, -0x1.6428b3546ce13p-55, \
    0x1.426b7e69ee697p-2, -0x1.f09c75705c59fp-56, 0x1.e5f54b436e9d0p-1, 0x1.7eb0fd02fc8bcp-55, \
    0x1.4a00c9b0f3d20p-2, 0x1.823ba6bb08eadp-56, 0x1.e4af14b2a449cp-1, -0x1.68ca02e8a6833p-55, \
    0x1.5190ecf68a77ap-2, 0x1.b357155eef0f3p-56, 0x1.e3614b680d6a5p-1, -0x1.27793aa015237p-56, \
    0x1.591bc9fa2f597p-2, 0x1.7c74bac3fe0cbp-57, 0x1.e20bf49acd6c1p-1, -0x1.660aec7ef636bp-58, \
    0x1.60a1429078775p-2, 0x1.b1fd80ba89133p-58, 0x1.e0af15a03dbcep-1, 0x1.fe8e702771ae6p-58, \
    0x1.682138a38d7f7p-2, -0x1.d889202444aadp-56, 0x1.df4ab3ebd875ep-1, -0x1.e2d8a7e6736c4p-55, \
    0x1.6f9b8e33a0255p-2, 0x1.42bc14ee9da0dp-56, 0x1.ddded50f228d6p-1, -0x1.e80c8d42ba2bfp-57, \
    0x1.7710255764214p-2, -0x1.6ead7314bb6cep-57, 0x1.dc6b7eb995912p-1, 0x1.4b364776dcd35p-58, \
    0x1.7e7ee03c86d4ep-2, -0x1.b63bcdabf5af2p-56, 0x1.daf0b6b888e83p-1, 0x1.a249e2b5e5ceap-55, \
    0x1.85e7a12826949p-2, 0x1.8a40e9b5face0p-56, 0x1.d96e82f71a9dcp-1, 0x1.ff61bd5d2039dp-55, \
    0x1.8d4a4a774992fp-2, 0x1.44a02ea766326p-56, 0x1.d7e4e97e17b4ap-1, -0x1.3b770352bed94p-57, \
    0x1.94a6be9f546c5p-2, -0x1.69ce13e683f58p-56, 0x1.d653f073e4040p-1, -0x1.76236434bec37p-55, \
    0x1.9bfce02e80510p-2, 0x1.09e39a320b0a4p-56, 0x1.d4bb9e1c619e0p-1, 0x1.f34bb77858f61p-55, \
    0x1.a34c91cc50ccap-2, -0x1.a310e3b50cecdp-58, 0x1.d31bf8d8d7c06p-1, 0x1.e60dd3089cbddp-56, \
    0x1.aa95b63a09277p-2, -0x1.6293eb13c0381p-57, 0x1.d1750727d94f0p-1, 0x1.0d52b1ec1a48ep-55, \
    0x1.b1d8305321617p-2, -0x1.ae242cb99f519p-56, 0x1.cfc6cfa52ad9fp-1, 0x1.8b5b5508f2a0dp-55, \
    0x1.b913e30dbac43p-2, -0x1.e38ad2f6c3ff1p-56, 0x1.ce115909a82e5p-1, 0x1.1f139bb31109ap-55, \
    0x1.c048b17b140a3p-2, 0x1.19fe6757e9fa7p-57, 0x1.cc54aa2b2972ep-1, 0x1.4ee162ba83a98p-57, \
    0x1.c7767ec7fd19ep-2, -0x1.eb14d1a3d5826p-58, 0x1.ca90c9fc67d0bp-1, -0x1.46a81485e3462p-57, \
    0x1.ce9d2e3d4a51fp-2, -0x1.2fc8a12dae298p-57, 0x1.c8c5bf8ce1a84p-1, 0x1.ab3d1a1590123p-56, \
    0x1.d5bca34047661p-2, 0x1.28a44a75fc29cp-56, 0x1.c6f39208be53bp-1, -0x1.741dbfbaadb42p-55, \
    0x1.dcd4c15329c9ap-2, 0x1.0d4c6e171fd9ap-56, 0x1.c51a48b8b175ep-1, -0x1.1bbb43b9aa880p-57, \
    0x1.e3e56c1582a69p-2, -0x1.0a4821099f88fp-58, 0x1.c339eb01ddd81p-1, -0x1.caaf5ee82c5c0p-55, \
    0x1.eaee8744b05f0p-2, -0x1.789b43c9b027dp-58, 0x1.c1528065b7d50p-1, -0x1.892111312e828p-55, \
    0x1.f1eff6bc4f97bp-2, 0x1.17212f8a7525cp-56, 0x1.bf641081e7536p-1, 0x1.b7bd71628a9a1p-55, \
    0x1.f8e99e76abc97p-2, 0x1.9d950af2d00a3p-58, 0x1.bd6ea310294f5p-1, 0x1.31bbcc88c109dp-56, \
    0x1.ffdb628d2f57ap-2, 0x1.f4a992e905b6ap-57, 0x1.bb723fe630f32p-1, 0x1.72bd2452d0a39p-56, \
    0x1.0362939c69955p-1, -0x1.2d8cd78397b01p-55, 0x1.b96eeef58840ep-1, 0x1.45a3cc78fade0p-58, \
    0x1.06d3686946e5bp-1, 0x1.3f5ae4538ff1bp-55, 0x1.b764b84b704c2p-1, -0x1.f5848c21b389bp-55, \
    0x1.0a4021e9e1001p-1, -0x1.6f643a13914f6p-55, 0x1.b553a410c104ep-1, 0x1.8ff7947027a15p-58, \
    0x1.0da8b26b5672ep-1, -0x1.a58def0bee909p-55, 0x1.b33bba89c8948p-1, 0x1.ea6a51d1f6ca9p-55, \
    0x1.110d0c4b69c3bp-1, 0x1.d918998809981p-55, 0x1.b11d04162a4c6p-1, 0x1.1dd561efbc0c2p-56, \
    0x1.146d21f8b7f82p-1, 0x1.bf9535e2739a8p-56, 0x1.aef78930bd275p-1, -0x1.f836279746f94p-56, \
    0x1.17c8e5f2eedb0p-1, 0x1.35e57102e2488p-57, 0x1.accb526f69de5p-1, 0x1.8fb6a8dd6b6ccp-55, \
    0x1.1b204acb02fddp-1, -0x1.f190c70cbb5fep-58, 0x1.aa98688308913p-1, -0x1.b83d607cd5072p-63, \
    0x1.1e7343236574cp-1, 0x1.22a3fa4f41d5ap-56, 0x1.a85ed4373e02dp-1, 0x1.9be06385ec792p-57, \
    0x1.21c1c1b0394cfp-1, 0x1.e5b324b23aa31p-58, 0x1.a61e9e72586afp-1, 0x1.58330e2fd453fp-55, \
    0x1.250bb93788bbbp-1, 0x1.ea3d02457bccep-56, 0x1.a3d7d0352bdcfp-1, -0x1.68dbaeca19669p-55, \
    0x1.28511c917a067p-1, -0x1.01df1d9a16b70p-55, 0x1.a18a729aee445p-1, 0x1.95e25736c0357p-60, \
    0x1.2b91dea88421ep-1, -0x1.fa371db216ab0p-55, 0x1.9f368ed912f85p-1, -0x1.1d200c5791606p-55, \
    0x1.2ecdf279a3082p-1, 0x1.d3557e0e7e37ep-55, 0x1.9cdc2e3f25e5cp-1, 0x1.3f99112993f62p-55, \
    0x1.32054b148bc4fp-1, 0x1.f6b42095a135bp-55, 0x1.9a7b5a36a6514p-1, 0x1.722cfcc9fa7a9p-55, \
    0x1.3537db9be0367p-1, 0x1.b327e7af040f0p-57, 0x1.98141c42e1310p-1, 0x1.d1ff80488f08dp-55, \
    0x1.386597456282bp-1, -0x1.10fada93b07a8p-56, 0x1.95a67e00cb1fdp-1, -0x1.0befda21f862dp-55, \
    0x1.3b8e715a2840ap-1, -0x1.97653a7d2f07ap-56, 0x1.93328926d9e92p-1, -0x1.bb77003600cdap-55, \
    0x1.3eb25d36cd53ap-1, -0x1.be570e1570fc0p-58, 0x1.90b84784ddaf7p-1, -0x1.0feb10ab93b87p-56, \
    0x1.41d14e4ba6790p-1, 0x1.4608fd287ecf5p-55, 0x1.8e37c303d9ad1p-1, -0x1.463a4b53d4bf8p-57, \
    0x1.44eb381cf386bp-1, -0x1.3ed6c1e6a5505p-55, 0x1.8bb105a5dc900p-1, 0x1.863e03e9474c1p-55, \
    0x1.48000e431159fp-1, -0x1.b194a7463ed10p-55, 0x1.89241985d871fp-1, 0x1.c48d9c413ed84p-55, \
    0x1.4b0fc46aab761p-1, 0x1.0da05738cc59cp-61, 0x1.869108d77a6c6p-1, 0x1.338ffe2bfe9ddp-56, \
    0x1.4e1a4e54ed51bp-1, -0x1.a492f89b7c76ap-55, 0x1.83f7dde701ca0p-1, -0x1.152cf609bc6e8p-59, \
    0x1.511f9fd7b351cp-1, -0x1.5c0e861c48831p-55, 0x1.8158a31916d5dp-1, -0x1.de8b90b8228dep-57, \
    0x1.541facddbb724p-1, 0x1.232c28520d391p-56, 0x1.7eb362eaa1488p-1, 0x1.a1d65a4a5959fp-58, \
    0x1.571a6966d59b3p-1, 0x1.c843b4d0fb197p-58, 0x1.7c0827f09e54fp-1, -0x1.c73d6d72aee68p-57, \
    0x1.5a0fc98813a12p-1, -0x1.d82e2b7d4227bp-55, 0x1.7956fcd7f6543p-1, -0x1.ab276e9d45ae4p-55, \
    0x1.5cffc16bf8f0dp-1, 0x1.96cb370eb578ap-55, 0x1.769fec655211fp-1, -0x1.827d5cf8c68c5p-57, \
    0x1.5fea4552a9e57p-1, 0x1.0b6cef7ee20b7p-55, 0x1.73e30174efba1p-1, -0x1.5d3ae3d94ad5fp-57, \
    0x1.62cf49921ac79p-1, -0x1.edd9855b6241ap-55, 0x1.712046fa77678p-1, 0x1.425b0a5029c81p-55, \
    0x1.65aec2963e755p-1, 0x1.126f96b71053cp-55, 0x1.6e57c800cf55ep-1, 0x1.60286dedbd0a6p-55, \
    0x1.6888a4e134b2fp-1, -0x1.6b7d37644d5e6p-55, 0x1.6b898fa9efb5dp-1, 0x1.15ac786ccf4b2p-56, \
    0x1.6b5ce50b7821ap-1, -0x1.5d5158f702e0fp-57, 0x1.68b5a92eb6253p-1, -0x1.9a91ad985f89cp-55,

/* series coefficients: S_n = (-1)^n/(2n+1)!, C_n = (-1)^n/(2n)!, A_n = (-1)^n/(2n+1) */
#define LIFE_CR_S1H -0x1.5555555555555p-3
#define LIFE_CR_S1L -0x1.5555555555555p-57
#define LIFE_CR_C1H -0x1.0000000000000p-1
#define LIFE_CR_C1L 0.0
#define LIFE_CR_A1H -0x1.5555555555555p-2
#define LIFE_CR_A1L -0x1.5555555555555p-56
#define LIFE_CR_S2H 0x1.1111111111111p-7
#define LIFE_CR_S2L 0x1.1111111111111p-63
#define LIFE_CR_C2H 0x1.5555555555555p-5
#define LIFE_CR_C2L 0x1.5555555555555p-59
#define LIFE_CR_A2H 0x1.999999999999ap-3
#define LIFE_CR_A2L -0x1.999999999999ap-57
#define LIFE_CR_S3H -0x1.a01a01a01a01ap-13
#define LIFE_CR_S3L -0x1.a01a01a01a01ap-73
#define LIFE_CR_C3H -0x1.6c16c16c16c17p-10
#define LIFE_CR_C3L 0x1.f49f49f49f49fp-65
#define LIFE_CR_A3H -0x1.2492492492492p-3
#define LIFE_CR_A3L -0x1.2492492492492p-57
#define LIFE_CR_S4H 0x1.71de3a556c734p-19
#define LIFE_CR_S4L -0x1.c154f8ddc6c00p-73
#define LIFE_CR_C4H 0x1.a01a01a01a01ap-16
#define LIFE_CR_C4L 0x1.a01a01a01a01ap-76
#define LIFE_CR_A4H 0x1.c71c71c71c71cp-4
#define LIFE_CR_A4L 0x1.c71c71c71c71cp-58
#define LIFE_CR_S5H -0x1.ae64567f544e4p-26
#define LIFE_CR_S5L 0x1.c062e06d1f209p-80
#define LIFE_CR_C5H -0x1.27e4fb7789f5cp-22
#define LIFE_CR_C5L -0x1.cbbc05b4fa99ap-76
#define LIFE_CR_A5H -0x1.745d1745d1746p-4
#define LIFE_CR_A5L 0x1.745d1745d1746p-59
/* pi/2 = P1 + P2 + P3 + P4 (P1..P3 have 33 significant bits) */
#define LIFE_CR_PIO2_1 0x1.921fb54400000p+0
#define LIFE_CR_PIO2_2 0x1.0b4611a600000p-34
#define LIFE_CR_PIO2_3 0x1.3198a2e000000p-69
#define LIFE_CR_PIO2_4 0x1.b839a252049c1p-104
#define LIFE_CR_TWO_OVER_PI 0x1.45f306dc9c883p-1
#define LIFE_CR_PIO2_H 0x1.921fb54442d18p+0
#define LIFE_CR_PIO2_L 0x1.1a62633145c07p-54
#define LIFE_CR_PI_H 0x1.921fb54442d18p+1
#define LIFE_CR_PI_L 0x1.1a62633145c07p-53
#define LIFE_CR_PIO4_H 0x1.921fb54442d18p-1
#define LIFE_CR_PIO4_L 0x1.1a62633145c07p-55
#define LIFE_CR_TPIO4_H 0x1.2d97c7f3321d2p+1
#define LIFE_CR_TPIO4_L 0x1.a79394c9e8a0ap-54

#endif

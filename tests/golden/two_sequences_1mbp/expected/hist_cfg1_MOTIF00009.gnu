set output "hist_cfg1_MOTIF00009.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-56.3627:16.7501]
set yrange [0:142475]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00009.dat" using 1:2 title 'MOTIF00009 (cfg1)' with boxes

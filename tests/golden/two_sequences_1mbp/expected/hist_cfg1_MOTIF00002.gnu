set output "hist_cfg1_MOTIF00002.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-49.4068:10.9065]
set yrange [0:126365]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00002.dat" using 1:2 title 'MOTIF00002 (cfg1)' with boxes
